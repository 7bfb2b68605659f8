// punc_gpu.hpp - C++ front end over the C ABI of punc_gpu.h with the names and
// argument order of the PUNC++ particle path, so a time loop written against
// the reference (interaction/interaction.cpp:342-480) keeps its shape:
//
//     punc::gpu::distribute_cg1(pop, rho, dv_inv);
//     poisson.solve_circuit(phi, rho, mesh, objects, circuit);
//     esolver.solve(E, phi);
//     KE = punc::gpu::boris(pop, E, B, dt);
//     punc::gpu::move(pop, dt);
//     pop.update(objects, dt);
//     punc::gpu::inject_particles(pop, species, dt, seed, n);
//
// DOLFIN types are replaced by plain arrays: a Mesh is built from vertex
// coordinates, cell vertex ids and tagged boundary facets; Functions are views
// of the fields the engine keeps on the device.  Errors throw punc::gpu::Error
// carrying the pg_status code.
#ifndef PUNC_GPU_HPP
#define PUNC_GPU_HPP

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <utility>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "punc_gpu.h"

namespace punc {
namespace gpu {

struct Error : std::runtime_error {
    int code;
    Error(int c, const char *msg) : std::runtime_error(std::string("punc_gpu: ") + (msg ? msg : "")), code(c) {}
};

inline void check(int rc) {
    if (rc != PG_OK) throw Error(rc, pg_last_error());
}

// Mesh (punc/include/punc/mesh.h:49-97) as arrays: tag 1 = exterior, 2.. = objects.
class Mesh {
public:
    Mesh(const std::vector<double> &coords, const std::vector<int64_t> &cells,
         const std::vector<int64_t> &bfacet_vertices, const std::vector<int32_t> &bfacet_tags,
         double eps0_ = 1.0, const std::vector<int64_t> *vertex_to_dof = nullptr, int64_t n_dofs = 0)
        : eps0(eps0_) {
        pg_mesh_desc d{};
        d.n_vertices = (int64_t)(coords.size() / 3);
        d.coords = coords.data();
        d.n_cells = (int64_t)(cells.size() / 4);
        d.cells = cells.data();
        d.n_boundary_facets = (int64_t)(bfacet_tags.size());
        d.bfacet_vertices = bfacet_vertices.data();
        d.bfacet_tags = bfacet_tags.data();
        d.n_dofs = vertex_to_dof ? n_dofs : d.n_vertices;
        d.vertex_to_dof = vertex_to_dof ? vertex_to_dof->data() : nullptr;
        check(pg_mesh_build(&d, eps0, &handle));
    }
    ~Mesh() { pg_mesh_free(handle); }
    Mesh(const Mesh &) = delete;
    Mesh &operator=(const Mesh &) = delete;
    std::size_t num_cells() const {
        const void *p = nullptr;
        int64_t n = 0;
        check(pg_mesh_array(handle, PG_T_VOLUME, &p, &n));
        return (std::size_t)n;
    }
    // Mesh::volume (punc/src/mesh.cpp:147-170): cell volumes summed in cell order.
    double volume() const {
        const void *p = nullptr;
        int64_t n = 0;
        check(pg_mesh_array(handle, PG_T_VOLUME, &p, &n));
        const double *v = static_cast<const double *>(p);
        double s = 0.0;
        for (int64_t c = 0; c < n; ++c) s += v[c];
        return s;
    }
    pg_mesh *handle = nullptr;
    double eps0;
};

// Object (punc/include/punc/object.h:80-130).
struct Object {
    explicit Object(std::size_t bnd_id_) : bnd_id(bnd_id_) {}
    void set_potential(double p) { potential = p; }
    double get_potential() const { return potential; }
    double charge = 0, current = 0;
    std::size_t bnd_id;
    double potential = 0;
};
using ObjectVector = std::vector<std::shared_ptr<Object>>;

struct VSource { int node_a, node_b; double value; };
struct ISource { int node_a, node_b; double value; };
using VSourceVector = std::vector<VSource>;
using ISourceVector = std::vector<ISource>;

// Maxwellian species of simulation particles (punc/src/population.cpp:41-70):
// q, m and n of a simulation particle and the velocity distribution; weight,
// num and debye as make_species derives them.
struct Species {
    double q, m, n, vth;
    double vd[3] = {0, 0, 0};
    double vdf_range = 5.0;
    double weight = 1.0;      // physical particles per simulation particle
    std::size_t num = 0;      // initial number of simulation particles
    double debye = 0.0;       // Debye length
};

// How the amount of simulation particles is given (punc/include/punc/population.h:50-55).
enum class ParticleAmountType { in_total, per_cell, per_volume, phys_per_sim };

// Species::Species (punc/src/population.cpp:41-70) with a Maxwellian velocity
// distribution of thermal speed vth and drift vd (Maxwellian::debye,
// punc/src/distributions.cpp:74-77); eps0 = 0 takes the mesh's.  The amount
// becomes physical particles per simulation particle through the reference's
// chain per cell -> in total -> per volume -> weight.
inline Species make_species(double charge, double mass, double density, double amount, ParticleAmountType type,
                            const Mesh &mesh, double vth, const double *vd = nullptr, double vdf_range = 5.0,
                            double eps0 = 0.0) {
    const double volume = mesh.volume();
    switch (type) {
    case ParticleAmountType::per_cell:
        amount *= (double)mesh.num_cells();
        [[fallthrough]];
    case ParticleAmountType::in_total:
        amount /= volume;
        [[fallthrough]];
    case ParticleAmountType::per_volume:
        amount = density / amount;
        [[fallthrough]];
    case ParticleAmountType::phys_per_sim:
        break;
    default:
        throw Error(PG_ERR_ARG, "make_species: invalid ParticleAmountType");
    }
    Species s{charge * amount, mass * amount, density / amount, vth};
    if (vd)
        for (int k = 0; k < 3; ++k) s.vd[k] = vd[k];
    s.vdf_range = vdf_range;
    s.weight = amount;
    s.num = (std::size_t)(s.n * volume);
    const double e0 = eps0 != 0.0 ? eps0 : mesh.eps0;
    s.debye = std::sqrt(e0 * s.m / (s.n * s.q * s.q)) * vth;
    return s;
}

// min_plasma_period (punc/src/population.cpp:72-80).
inline double min_plasma_period(const std::vector<Species> &species, double eps0) {
    double wp_max = 0;
    for (auto &s : species) {
        const double wp = std::sqrt(s.q * s.q * s.n / (eps0 * s.m));
        if (wp > wp_max) wp_max = wp;
    }
    return 2 * 3.14159265358979323846 / wp_max;
}

namespace detail {
inline std::vector<pg_object> to_c(const ObjectVector &objs) {
    std::vector<pg_object> v;
    for (auto &o : objs) v.push_back(pg_object{(int64_t)o->bnd_id, o->charge, o->current, o->potential});
    return v;
}
inline void from_c(const std::vector<pg_object> &v, ObjectVector &objs) {
    for (std::size_t k = 0; k < objs.size(); ++k) {
        objs[k]->charge = v[k].charge;
        objs[k]->current = v[k].current;
        objs[k]->potential = v[k].potential;
    }
}
}  // namespace detail

// Particle<len> (punc/include/punc/population.h:74-94): the 64-byte record
// {x, v, q, m} of a particle.
template <std::size_t len = 3>
struct Particle {
    double x[len];
    double v[len];
    double q;
    double m;
    Particle(const double *x_, const double *v_, double q_, double m_) : q(q_), m(m_) {
        for (std::size_t i = 0; i < len; ++i) {
            x[i] = x_[i];
            v[i] = v_[i];
        }
    }
    Particle() {}
};

template <std::size_t len> class Population;

// Population<3> (punc/include/punc/population.h:236-308) on the device.
template <> class Population<3> {
public:
    explicit Population(const Mesh &mesh, pg_config cfg = pg_config{}) {
        if (cfg.eps0 == 0) cfg.eps0 = mesh.eps0;
        check(pg_create(mesh.handle, &cfg, &handle));
    }
    ~Population() { pg_destroy(handle); }
    Population(const Population &) = delete;
    Population &operator=(const Population &) = delete;

    void add_particles(const std::vector<double> &xs, const std::vector<double> &vs, double q, double m) {
        int64_t added = 0;
        check(pg_add_particles(handle, xs.data(), vs.data(), (int64_t)(xs.size() / 3), q, m, &added));
    }
    // add_particles(const std::vector<Particle<len>> &) (population.h:437-446):
    // records outside the mesh are dropped; each run of consecutive records
    // with the same charge and mass goes in one call, so the engine's particle
    // ids follow the input order as the reference's cell vectors do.
    void add_particles(const std::vector<Particle<3>> &ps) {
        std::vector<double> xs, vs;
        std::size_t i = 0;
        while (i < ps.size()) {
            std::size_t j = i;
            xs.clear();
            vs.clear();
            while (j < ps.size() && ps[j].q == ps[i].q && ps[j].m == ps[i].m) {
                xs.insert(xs.end(), ps[j].x, ps[j].x + 3);
                vs.insert(vs.end(), ps[j].v, ps[j].v + 3);
                ++j;
            }
            add_particles(xs, vs, ps[i].q, ps[i].m);
            i = j;
        }
    }
    signed long int locate(const double *p) {
        int64_t c = -1;
        check(pg_locate(handle, p, 1, &c));
        return (signed long int)c;
    }
    void update(ObjectVector objects, double dt) {
        auto v = detail::to_c(objects);
        check(pg_update(handle, v.data(), (int32_t)v.size(), dt));
        detail::from_c(v, objects);
    }
    std::size_t num_of_particles() { return counts(0); }
    std::size_t num_of_negatives() { return counts(1); }
    std::size_t num_of_positives() { return counts(2); }
    // Population::statistics (population.h:746-805)
    void statistics(double *stats) { check(pg_statistics(handle, stats)); }
    // Population::save_file / load_file (population.h:806-878)
    void save_file(const std::string &fname, bool binary) { check(pg_population_save(handle, fname.c_str(), binary)); }
    void load_file(const std::string &fname, bool binary) {
        check(pg_population_load(handle, fname.c_str(), binary, nullptr));
    }

    pg_sim *handle = nullptr;
    static constexpr std::size_t g_dim = 3;

private:
    std::size_t counts(int which) {
        int64_t c[3] = {0, 0, 0};
        check(pg_num_particles(handle, &c[0], &c[1], &c[2]));
        return (std::size_t)c[which];
    }
};

// A field of the engine: E (DG0 vector), ECG1 (CG1 vector), rho or phi (CG1).
class Function {
public:
    enum Kind { E, ECG1, Rho, Phi };
    Function(Population<3> &pop, Kind k) : pop_(pop), kind_(k) {}
    std::vector<double> vector(std::size_t n) const {
        std::vector<double> out(n);
        if (kind_ == E) check(pg_get_efield(pop_.handle, out.data()));
        else if (kind_ == ECG1) check(pg_get_efield_cg1(pop_.handle, out.data()));
        else if (kind_ == Rho) check(pg_get_rho(pop_.handle, out.data()));
        else check(pg_get_phi(pop_.handle, out.data()));
        return out;
    }
    Population<3> &pop() const { return pop_; }

private:
    Population<3> &pop_;
    Kind kind_;
};

// pusher.h:66-130, 397-510, 648-681
inline double accel(Population<3> &pop, const Function &, double dt) {
    double ke = 0;
    check(pg_accel(pop.handle, dt, &ke));
    return ke;
}
inline double boris(Population<3> &pop, const Function &, const std::vector<double> &B, double dt) {
    double ke = 0;
    check(pg_boris(pop.handle, B.data(), dt, &ke));
    return ke;
}
// pusher.h:154-201, 282-372
inline double accel_cg1(Population<3> &pop, const Function &, double dt) {
    double ke = 0;
    check(pg_accel_cg1(pop.handle, dt, &ke));
    return ke;
}
inline double boris_cg1(Population<3> &pop, const Function &, const std::vector<double> &B, double dt) {
    double ke = 0;
    check(pg_boris_cg1(pop.handle, B.data(), dt, &ke));
    return ke;
}
inline void move(Population<3> &pop, double dt) { check(pg_move(pop.handle, dt)); }
inline void move_periodic(Population<3> &pop, double dt, const std::vector<double> &Ld) {
    check(pg_move_periodic(pop.handle, dt, Ld.data()));
}
// element_volume (punc/src/distributor.cpp:35-69): per dof, (d + 1) over the
// volume of its cells (voronoi) or one over that volume; the engine keeps the
// first as a mesh table, and the second is it divided by 4 (exact).
inline std::vector<double> element_volume(const Mesh &mesh, bool voronoi = true) {
    const void *p = nullptr;
    int64_t n = 0;
    check(pg_mesh_array(mesh.handle, PG_T_DV_INV, &p, &n));
    const double *dv = static_cast<const double *>(p);
    std::vector<double> out(dv, dv + n);
    if (!voronoi)
        for (auto &x : out) x /= 4.0;
    return out;
}
// distributor.h:168-210; dv_inv is the engine's own element_volume table.
inline void distribute_cg1(Population<3> &pop, Function &, const std::vector<double> &) {
    check(pg_distribute_cg1(pop.handle, nullptr));
}
inline double kinetic_energy(Population<3> &pop) {
    double ke = 0;
    check(pg_kinetic_energy(pop.handle, &ke));
    return ke;
}

// diagnostics.h:379-412, 433-465, 492-555
inline double particle_potential_energy_cg1(Population<3> &pop, const Function &) {
    double pe = 0;
    check(pg_potential_energy(pop.handle, &pe));
    return pe;
}
inline void density_cg1(Population<3> &pop, double weight_e, double weight_i, std::vector<double> &ne,
                        std::vector<double> &ni) {
    check(pg_density_cg1(pop.handle, weight_e, weight_i, ne.data(), ni.data()));
}
inline void density_dg0(Population<3> &pop, double weight_e, double weight_i, std::vector<double> &ne,
                        std::vector<double> &ni) {
    check(pg_density_dg0(pop.handle, weight_e, weight_i, ne.data(), ni.data()));
}

// State (punc/src/diagnostics.cpp:40-68): the resume file.
class State {
public:
    explicit State(std::string fname) : fname_(std::move(fname)) {}
    void save(std::size_t n, double t, const ObjectVector &objects) const {
        std::FILE *f = std::fopen(fname_.c_str(), "w");
        if (!f) throw std::runtime_error("State: cannot open " + fname_);
        std::fprintf(f, "%zu\t%g\t", n + 1, t);
        for (auto &o : objects) std::fprintf(f, "%g\t%g\n", o->charge, o->current);
        std::fclose(f);
    }
    void load(std::size_t &n, double &t, ObjectVector &objects) const {
        std::FILE *f = std::fopen(fname_.c_str(), "r");
        if (!f) throw std::runtime_error("State: cannot open " + fname_);
        char buf[4096] = {0};
        if (!std::fgets(buf, sizeof(buf), f)) buf[0] = 0;
        std::fclose(f);
        char *s = buf;
        n = std::strtoul(s, &s, 10);
        t = std::strtod(s, &s);
        for (auto &o : objects) {
            o->charge = std::strtod(s, &s);
            o->current = std::strtod(s, &s);
        }
    }

private:
    std::string fname_;
};

// History (punc/src/diagnostics.cpp:70-140, diagnostics.h:119-168): the
// history.dat preamble and rows in the reference's format.
class History {
public:
    History(const std::string &fname, std::size_t n_objects, std::size_t dim, bool stats,
            bool continue_simulation = false)
        : stats_(stats), f_(std::fopen(fname.c_str(), continue_simulation ? "a" : "w")) {
        if (!f_) throw std::runtime_error("History: cannot open " + fname);
        if (continue_simulation) return;
        std::fprintf(f_, "#:xaxis\tt\n#:name\tn\tt\tne\tni\tKE\tPE");
        for (std::size_t i = 0; i < n_objects; ++i) std::fprintf(f_, "\tV[%zu]\tI[%zu]\tQ[%zu]", i, i, i);
        if (stats) std::fprintf(f_, "\tmean_e\tstdev_e\tmean_i\tstdev_i");
        std::fprintf(f_, "\n#:long\ttimestep\ttime\t\"number of electrons\"\t\"number of ions\"\t"
                         "\"kinetic energy\"\t\"potential energy\"");
        for (std::size_t i = 0; i < n_objects; ++i) std::fprintf(f_, "\tvoltage\tcurrent\tcharge");
        if (stats)
            std::fprintf(f_, "\tmean velocity of electrons\tstandard deviation of electron velocities"
                             "\tmean velocity of ions\tstandard deviation of ion velocities");
        std::fprintf(f_, "\n#:units\t1\ts\tm**(-3)\tm**(-3)\tJ\tJ");
        const char *ui = dim == 1 ? "A/m**2" : dim == 2 ? "A/m" : "A";
        for (std::size_t i = 0; i < n_objects; ++i) std::fprintf(f_, "\tV\t%s\tC", ui);
        if (stats) std::fprintf(f_, "\tm/s\tm/s\tm/s\tm/s");
        std::fprintf(f_, "\n");
    }
    ~History() { if (f_) std::fclose(f_); }
    History(const History &) = delete;
    History &operator=(const History &) = delete;
    void save(std::size_t n, double t, double num_e, double num_i, double KE, double PE, const ObjectVector &objects,
              Population<3> &pop) {
        std::fprintf(f_, "%zu\t%.16e\t%.16e\t%.16e\t%.16e\t%.16e", n, t, num_e, num_i, KE, PE);
        for (auto &o : objects) std::fprintf(f_, "\t%.16e\t%.16e\t%.16e", o->potential, o->current, o->charge);
        if (stats_) {
            double st[4];
            pop.statistics(st);
            for (double v : st) std::fprintf(f_, "\t%.16e", v);
        }
        std::fprintf(f_, "\n");
    }

private:
    bool stats_;
    std::FILE *f_;
};

// EFieldDG0 (punc/src/efield.cpp:77-99)
struct EFieldDG0 {
    void solve(Function &E, const Function &) { check(pg_efield_dg0(E.pop().handle, nullptr)); }
};

// ESolver (punc/src/efield.cpp:41-75): CG1 projection of -grad(phi)
struct ESolver {
    void solve(Function &E, const Function &) { check(pg_esolver_solve(E.pop().handle, nullptr, nullptr)); }
};

// CircuitCM (punc/src/object_CM.cpp:135-197)
class CircuitCM {
public:
    CircuitCM(Population<3> &pop, ObjectVector &, const VSourceVector &vs, const ISourceVector &is, double dt) {
        std::vector<pg_source> v, i;
        for (auto &s : vs) v.push_back(pg_source{s.node_a, s.node_b, s.value});
        for (auto &s : is) i.push_back(pg_source{s.node_a, s.node_b, s.value});
        check(pg_circuit_cm_setup(pop.handle, v.data(), (int32_t)v.size(), i.data(), (int32_t)i.size(), dt));
    }
    bool correction_required = true;
};

// PoissonSolver (punc/src/poisson.cpp:260-385)
class PoissonSolver {
public:
    explicit PoissonSolver(Population<3> &pop) : pop_(pop) {}
    void solve(Function &, const Function &, ObjectVector &objects) {
        auto v = detail::to_c(objects);
        check(pg_poisson_solve(pop_.handle, v.data(), (int32_t)v.size(), nullptr, &info));
    }
    void solve_circuit(Function &, const Function &, const Mesh &, ObjectVector &objects, CircuitCM &) {
        auto v = detail::to_c(objects);
        check(pg_solve_circuit(pop_.handle, v.data(), (int32_t)v.size(), nullptr, &info));
        detail::from_c(v, objects);
    }
    pg_solve_info info{};

private:
    Population<3> &pop_;
};

// create_flux / inject_particles (punc/src/injector.cpp:104-171, injector.h:157-232)
inline void create_flux(Population<3> &pop, const std::vector<Species> &species) {
    std::vector<pg_species> s;
    for (auto &x : species) s.push_back(pg_species{x.q, x.m, x.n, x.vth, {x.vd[0], x.vd[1], x.vd[2]}, x.vdf_range});
    check(pg_create_flux(pop.handle, s.data(), (int32_t)s.size()));
}
inline std::size_t inject_particles(Population<3> &pop, const std::vector<Species> &, double dt, uint64_t seed,
                                    uint64_t step) {
    int64_t n = 0;
    check(pg_inject(pop.handle, dt, seed, step, &n));
    return (std::size_t)n;
}

// Extensions without a reference counterpart (the C ABI's pg_run_steps,
// pg_autotune, pg_amg_*, pg_get_phi_async and pg_adjoint_*), with the shim's
// object conventions.

// n_steps fused steps with the bookkeeping on the device, replaying a
// captured CUDA graph per step when `graph`; one result per step.
inline std::vector<pg_step_result> run_steps(Population<3> &pop, ObjectVector &objects, const pg_step_args &args,
                                             int32_t n_steps, bool graph = true) {
    auto v = detail::to_c(objects);
    std::vector<pg_step_result> res((std::size_t)std::max<int32_t>(1, n_steps));
    check(pg_run_steps(pop.handle, &args, v.data(), (int32_t)v.size(), n_steps, graph ? 1 : 0, res.data()));
    detail::from_c(v, objects);
    res.resize((std::size_t)std::max<int32_t>(0, n_steps));
    return res;
}

// Launch configuration and cell-sort interval chosen from timed real steps
// (the steps advance the simulation).
inline pg_tuning autotune(Population<3> &pop, ObjectVector &objects, const pg_step_args &args,
                          int32_t steps_per_trial = 2) {
    auto v = detail::to_c(objects);
    pg_tuning t{};
    check(pg_autotune(pop.handle, &args, v.data(), (int32_t)v.size(), steps_per_trial, &t));
    detail::from_c(v, objects);
    return t;
}

// AMG strength threshold of the Poisson preconditioner: set (rebuilds the
// hierarchy), or chosen from timed real steps among the candidates ({0, 0.01,
// 0.02} when empty; the steps advance the simulation), returning the choice.
inline void set_amg_strength(Population<3> &pop, double theta) { check(pg_amg_set_strength(pop.handle, theta)); }
inline double autotune_amg(Population<3> &pop, ObjectVector &objects, const pg_step_args &args,
                           int32_t steps_per_trial = 6, const std::vector<double> &thetas = {}) {
    auto v = detail::to_c(objects);
    double best = 0.0, ms = 0.0;
    check(pg_autotune_amg(pop.handle, &args, v.data(), (int32_t)v.size(), steps_per_trial,
                          thetas.empty() ? nullptr : thetas.data(), (int32_t)thetas.size(), &best, &ms));
    detail::from_c(v, objects);
    return best;
}

// The potential read back without waiting (pg_get_phi_async): `out` (ndof
// doubles, page-locked for the copy to overlap the next steps) holds it after
// synchronize(pop).
inline void get_phi_async(Population<3> &pop, double *out) { check(pg_get_phi_async(pop.handle, out)); }
inline void synchronize(Population<3> &pop) { check(pg_synchronize(pop.handle)); }

// Adjoint of K fused FP64 steps: forward (returns ||rho_K - target||^2), then
// the gradients with respect to the initial velocities and positions (by
// particle id), the uniform field E0 and the objects' fixed potentials.
struct AdjointGradients {
    std::vector<double> v0, x0, potentials;
    double E0[3] = {0, 0, 0};
};
inline double adjoint_forward(Population<3> &pop, ObjectVector &objects, const pg_step_args &args, int32_t n_steps,
                              int32_t ckpt_every, const std::vector<double> &rho_target) {
    auto v = detail::to_c(objects);
    double loss = 0;
    check(pg_adjoint_forward(pop.handle, &args, v.data(), (int32_t)v.size(), n_steps, ckpt_every, rho_target.data(),
                             &loss));
    return loss;
}
inline AdjointGradients adjoint_backward(Population<3> &pop, std::size_t n_particles, std::size_t n_objects) {
    AdjointGradients g;
    g.v0.assign(3 * n_particles, 0.0);
    g.x0.assign(3 * n_particles, 0.0);
    g.potentials.assign(n_objects, 0.0);
    check(pg_adjoint_backward(pop.handle, g.v0.data(), (int64_t)n_particles, g.E0, g.x0.data()));
    check(pg_adjoint_potential_gradient(pop.handle, g.potentials.data(), (int32_t)n_objects));
    return g;
}

}  // namespace gpu
}  // namespace punc

#endif  // PUNC_GPU_HPP
