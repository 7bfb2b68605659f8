/*
 * punc_gpu.h - C ABI of the GB300 particle-in-cell engine.
 *
 * Each entry point replaces one PUNC++ function or method on the
 * per-timestep particle path (paths are relative to the PUNC++ tree).
 * The engine owns every device buffer; host pointers passed in are
 * borrowed for the duration of the call only.  Every function returns a
 * pg_status; no function aborts, traps or exits.  A handle is not
 * thread-safe: calls on one handle are ordered on the handle's own CUDA
 * stream.
 */
#ifndef PUNC_GPU_H
#define PUNC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: pg_poisson_layout gained cycle_bytes; 3: pg_step_args.potential_energy
 * and pg_step_result.PE */
#define PG_ABI_VERSION 3

typedef enum pg_status {
    PG_OK = 0,
    PG_ERR_ARG = 1,            /* invalid argument or size */
    PG_ERR_CUDA = 2,           /* a CUDA runtime call failed */
    PG_ERR_MESH = 3,           /* inconsistent mesh: non-manifold facet, untagged boundary facet, degenerate cell */
    PG_ERR_CAPACITY = 4,       /* particle store full */
    PG_ERR_WALK_LIMIT = 5,     /* a relocation walk hit its step limit (cycle or non-finite position) */
    PG_ERR_NOT_CONVERGED = 6,  /* PCG reached its iteration cap */
    PG_ERR_STATE = 7,          /* call out of order (e.g. circuit or flux not set up) */
    PG_ERR_SINGULAR = 8        /* circuit matrix could not be inverted */
} pg_status;

typedef enum pg_precision {
    PG_FP64 = 0,   /* all particle arithmetic in FP64, reference rounding order */
    PG_MIXED = 1   /* FP32 particles, FP64 facet re-test, int64 fixed-point deposit */
} pg_precision;

/* Opaque handles. */
typedef struct pg_mesh pg_mesh;   /* host-side mesh tables */
typedef struct pg_sim pg_sim;     /* device-resident mesh, particles and solver */

/* Mesh as plain arrays, the content of a DOLFIN Mesh plus its facet
 * MeshFunction after Mesh::Mesh relabelled the tags
 * (punc/src/mesh.cpp:41-60): tag 1 = exterior boundary, 2.. = objects.
 * Every boundary facet must be listed with a tag >= 1. */
typedef struct pg_mesh_desc {
    int64_t n_vertices;
    const double *coords;            /* [n_vertices][3] */
    int64_t n_cells;
    const int64_t *cells;            /* [n_cells][4] vertex ids, any order */
    int64_t n_boundary_facets;
    const int64_t *bfacet_vertices;  /* [n_boundary_facets][3] */
    const int32_t *bfacet_tags;      /* [n_boundary_facets] */
    int64_t n_dofs;                  /* CG1 dofs; = n_vertices unless periodic */
    const int64_t *vertex_to_dof;    /* [n_vertices] or NULL (identity) */
} pg_mesh_desc;

/* Which host table pg_mesh_array returns. */
typedef enum pg_mesh_table {
    PG_T_CELL_VERTICES = 0,  /* int64 [Nc][4], ascending vertex ids (UFC order) */
    PG_T_BARYCENTRIC = 1,    /* double [Nc][12], rows 0-2 of the barycentric matrix */
    PG_T_PLANES = 2,         /* double [Nc][16], per facet i: -n.m, n_x, n_y, n_z */
    PG_T_NEIGHBOURS = 3,     /* int64 [Nc][4], neighbour across facet i or -tag */
    PG_T_CELL_DOFS = 4,      /* int64 [Nc][4] */
    PG_T_VOLUME = 5,         /* double [Nc] */
    PG_T_DV_INV = 6,         /* double [Ndof], (d+1) / patch volume */
    PG_T_CSR_ROWPTR = 7,     /* int64 [Ndof+1] */
    PG_T_CSR_COL = 8,        /* int64 [nnz] */
    PG_T_STIFFNESS = 9,      /* double [nnz], eps0 * P1 stiffness, no boundary conditions */
    PG_T_MASS = 10,          /* double [nnz], consistent P1 mass */
    PG_T_EXT_FACETS = 11,    /* double [Nf][14]: area, 9 vertex coords, 3 inward normal, cell */
    PG_T_BC_KIND = 12,       /* int64 [Ndof]: -1 free, 0 exterior, k>=1 object k (tag k+1) */
    PG_T_OBJ_FACETS = 13     /* double [No][7]: cell, object index, area, 3 outward normal, local facet */
} pg_mesh_table;

typedef struct pg_config {
    int32_t precision;          /* pg_precision */
    int32_t periodic;           /* 1: remove the constant null space (no Dirichlet BC) */
    double eps0;                /* vacuum permittivity in simulation units */
    int64_t particle_capacity;  /* particle slots to allocate (0: automatic) */
    int32_t max_walk_steps;     /* relocation walk step limit (0: 100000) */
    int32_t sort_interval;      /* cell-sort period in steps of pg_step (0: 20) */
    double pcg_rtol;            /* 0: 1e-12, PoissonSolver default (punc/src/poisson.cpp:326-328) */
    double pcg_atol;            /* 0: 1e-14 */
    int32_t pcg_max_iter;       /* 0: 1000 */
    int32_t pcg_warm_start;     /* 1: start PCG from the previous potential; 2: from the linear
                                   extrapolation 2 phi_n - phi_(n-1) of the last two */
    double ext_E[3];            /* exterior Dirichlet value phi = x . ext_E (PhiBoundary) */
    int32_t circuit_resolve;    /* 1: CircuitCM correction by a second solve, as the reference
                                   (punc/src/poisson.cpp:373-375); 0: by superposition of the
                                   unit-potential Laplace solutions kept from set-up (same
                                   potential up to the solver tolerance, one solve per step) */
    int32_t pcg_precision;      /* Jacobi preconditioner only: 0: FP64 PCG for PG_FP64, mixed PCG
                                   for PG_MIXED; 1: FP64 PCG; 2: mixed PCG (FP32 recurrence, FP64
                                   solution, inner products and true-residual replacement; same
                                   FP64 stopping test) */
    int32_t pcg_precond;        /* 0: smoothed-aggregation AMG V-cycle (mixed PCG; the reference
                                   preconditions with hypre AMG, punc/src/object_CM.cpp:208-219);
                                   1: Jacobi */
} pg_config;

/* Reference Object (punc/include/punc/object.h:80-130). */
typedef struct pg_object {
    int64_t bnd_id;     /* boundary tag, 2 = first object */
    double charge;
    double current;
    double potential;
} pg_object;

/* Reference VSource / ISource (punc/include/punc/object.h:45-71). */
typedef struct pg_source {
    int32_t node_a;     /* -1 = ground */
    int32_t node_b;
    double value;
} pg_source;

/* Species with a Maxwellian velocity distribution
 * (punc/src/population.cpp:41-70, punc/src/distributions.cpp:23-77). */
typedef struct pg_species {
    double q;           /* charge of a simulation particle */
    double m;           /* mass of a simulation particle */
    double n;           /* number density of simulation particles */
    double vth;         /* thermal speed */
    double vd[3];       /* drift velocity */
    double vdf_range;   /* rejection box half-width in vth (0: 5) */
} pg_species;

typedef struct pg_solve_info {
    int32_t iterations;
    int32_t solves;
    double residual;    /* final ||r||_2 of the last solve */
    double rhs_norm;    /* ||b||_2 of the last solve */
} pg_solve_info;

/* One fused timestep in the order of the time loop of
 * interaction/interaction.cpp:342-480. */
typedef struct pg_step_args {
    double dt;
    double B[3];             /* uniform magnetic field */
    int32_t first_step;      /* 1: push with dt/2 (leapfrog start) */
    int32_t use_accel;       /* 1: accel() instead of boris() */
    int32_t periodic_move;   /* 1: move_periodic with Ld */
    double Ld[3];
    int32_t inject;          /* 1: flux injection after update */
    uint64_t seed;           /* injection RNG key */
    uint64_t step;           /* injection RNG counter (time step number) */
    double E0[3];            /* uniform external field added to the cell (or vertex) field */
    int32_t efield_cg1;      /* 1: CG1 field by ESolver and accel_cg1 / boris_cg1, the reference
                                time loop's default (interaction/interaction.cpp:361-389);
                                0: DG0 field (EFieldDG0) and accel / boris */
    int32_t potential_energy; /* 1: pg_step returns the potential energy of the particles at the
                                step's start in the step's potential, where the time loop takes
                                it (particle_potential_energy_cg1 after the field,
                                interaction/interaction.cpp:367-372); pg_run_steps refuses it */
} pg_step_args;

typedef struct pg_step_result {
    double KE;               /* kinetic energy at mid-step (returned by the push) */
    int64_t n_particles;     /* after injection */
    int64_t n_absorbed;
    int64_t n_injected;
    int32_t pcg_iterations;  /* summed over the step's solves */
    double pcg_residual;
    double PE;               /* potential energy when pg_step_args.potential_energy = 1, else 0 */
} pg_step_result;

/* ---- library ---------------------------------------------------------- */
int32_t pg_abi_version(void);
const char *pg_last_error(void);       /* thread-local text of the last failure */
/* One block of the Philox4x32-10 generator behind pg_inject (the reference's
 * std::mt19937_64, punc/include/punc/injector.h:161, is unseeded and cannot be
 * reproduced; this stream can).  No GPU needed. */
int pg_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ---- mesh tables (host only, no GPU needed) ---------------------------- */
/* Population<3>::Population + init_localizer + Cell::init_barycentric_matrix
 * (punc/include/punc/population.h:310-389, punc/src/population.cpp:181-240),
 * element_volume (punc/src/distributor.cpp:35-69), P1 stiffness and mass
 * (punc/ufl/Potential3D.ufl), Mesh::exterior_boundaries
 * (punc/src/mesh.cpp:166-236). */
int pg_mesh_build(const pg_mesh_desc *desc, double eps0, pg_mesh **out);
int pg_mesh_array(const pg_mesh *mesh, int32_t which, const void **data, int64_t *count);
int pg_mesh_free(pg_mesh *mesh);

/* ---- engine ------------------------------------------------------------ */
int pg_create(const pg_mesh *mesh, const pg_config *cfg, pg_sim **out);
int pg_destroy(pg_sim *sim);
int pg_status_detail(pg_sim *sim, int32_t *code, int64_t *index);

/* Population::add_particles(xs, vs, q, m) (punc/include/punc/population.h:411-435):
 * locate each point and keep those inside the mesh. */
int pg_add_particles(pg_sim *sim, const double *xs, const double *vs, int64_t n,
                     double q, double m, int64_t *n_added);
/* pg_add_particles locating only in cells [cell_lo, cell_hi): batched runs keep
 * each run's mesh at its own coordinates (the runs overlap in space) and load
 * each run's particles into its own cell range. */
int pg_add_particles_range(pg_sim *sim, const double *xs, const double *vs, int64_t n, double q, double m,
                           int32_t cell_lo, int32_t cell_hi, int64_t *n_added);
/* Batched runs: per exterior facet (engine order, PG_T_EXT_FACETS rows) the
 * injection RNG stream id and seed offset, so that each run draws the streams
 * of its standalone mesh (facet j of run r: stream = j - first facet of r,
 * key = seed + offset of r).  Either array may be NULL (keep j / 0). */
int pg_set_injection_streams(pg_sim *sim, const uint32_t *facet_stream, const uint64_t *facet_seed);
/* num_of_particles / num_of_negatives / num_of_positives
 * (punc/include/punc/population.h:701-744). */
int pg_num_particles(pg_sim *sim, int64_t *total, int64_t *negatives, int64_t *positives);
/* Download live particles ordered by (cell, particle id).  Any output may be NULL. */
int pg_get_particles(pg_sim *sim, int64_t capacity, double *x, double *v, double *q,
                     double *m, int64_t *cell, int64_t *pid, int64_t *n_out);
/* Population::save_file / load_file (punc/include/punc/population.h:806-878):
 * binary = 64-byte {x[3], v[3], q, m} records, text = "%.17g" columns; cells in
 * order, by particle id inside a cell.  Loading adds the particles in file
 * order (ids follow the records, as the reference's one-by-one
 * add_particles), one pg_add_particles call per run of records with the same
 * q, m; n_added may be NULL. */
int pg_population_save(pg_sim *sim, const char *fname, int32_t binary);
int pg_population_load(pg_sim *sim, const char *fname, int32_t binary, int64_t *n_added);
/* Population::locate (punc/src/population.cpp:24-39), for n points. */
int pg_locate(pg_sim *sim, const double *xs, int64_t n, int64_t *cells);

/* Single-point walks of Population from given cells (no particles move):
 * mode 0 = relocate_fast (punc/include/punc/population.h:539-569, the first
 * facet with a positive plane value, the walk of update), mode 1 = relocate
 * and relocate_stat (population.h:454-538, the facet of the largest plane
 * value; the walk stays only when every value is negative).  cells_out[i] =
 * the final cell or -tag of the boundary hit; crossings (optional) = facets
 * crossed, relocate_stat's count.  A walk at the step limit gives
 * PG_ERR_WALK_LIMIT. */
int pg_relocate(pg_sim *sim, const double *xs, const int64_t *cells, int64_t n, int32_t mode, int64_t *cells_out,
                int32_t *crossings);

/* EFieldDG0::solve (punc/src/efield.cpp:95-99): E = -grad(phi) per cell.
 * phi may be NULL (use the device potential). */
int pg_efield_dg0(pg_sim *sim, const double *phi);
int pg_set_efield(pg_sim *sim, const double *E_cells);   /* [Nc][3] */
int pg_get_efield(pg_sim *sim, double *E_cells);         /* [Nc][3] */

/* accel with a DG0 field (punc/include/punc/pusher.h:66-130). */
int pg_accel(pg_sim *sim, double dt, double *KE);
/* boris with a DG0 field and uniform B (punc/include/punc/pusher.h:397-510). */
int pg_boris(pg_sim *sim, const double B[3], double dt, double *KE);
/* move / move_periodic (punc/include/punc/pusher.h:648-681). */
int pg_move(pg_sim *sim, double dt);
int pg_move_periodic(pg_sim *sim, double dt, const double Ld[3]);
/* Population::update (punc/include/punc/population.h:641-699): relocate every
 * particle by the facet walk of relocate_fast (539-569), absorb at boundaries,
 * zero then tally object currents, charge += current, current /= dt. */
int pg_update(pg_sim *sim, pg_object *objects, int32_t n_objects, double dt);
/* The absorbed-particle tally of the last pg_update, pg_step or pg_run_steps
 * step, per boundary tag and species: Population::update
 * (punc/include/punc/population.h:641-699) sums the same tally over the
 * species into each object's current.  counts[t * n_species + k] = particles
 * of species k absorbed at tag t (t = 0 .. n_tags-1; 1 = exterior boundary,
 * 2.. objects; n_tags <= 256), q[k] and m[k] the species' charge and mass, in
 * the engine's species order (first use of each (q, m)), for k < n_species;
 * *n_species_out = the number of species.  Any output may be NULL. */
int pg_absorbed_counts(pg_sim *sim, int64_t *counts, int32_t n_tags, int32_t n_species, double *q, double *m,
                       int32_t *n_species_out);
/* kinetic_energy (punc/include/punc/diagnostics.h:248-265). */
int pg_kinetic_energy(pg_sim *sim, double *KE);

/* distribute_cg1 (punc/include/punc/distributor.h:168-210): rho = dv_inv * sum q lambda.
 * rho may be NULL (keep it on the device only). */
int pg_distribute_cg1(pg_sim *sim, double *rho);
int pg_set_rho(pg_sim *sim, const double *rho);

/* PoissonSolver::solve (punc/src/poisson.cpp:343-362) with object potentials
 * as Dirichlet values; phi may be NULL. */
int pg_poisson_solve(pg_sim *sim, const pg_object *objects, int32_t n_objects,
                     double *phi, pg_solve_info *info);
/* CircuitCM::CircuitCM (punc/src/object_CM.cpp:135-197): capacitance matrix
 * by one Laplace solve per object, then the circuit matrix. */
int pg_circuit_cm_setup(pg_sim *sim, const pg_source *vsources, int32_t n_vsources,
                        const pg_source *isources, int32_t n_isources, double dt);
/* PoissonSolver::solve_circuit (punc/src/poisson.cpp:364-376) with CircuitCM
 * pre_solve / post_solve (punc/src/object_CM.cpp:53-60, 328-357). */
int pg_solve_circuit(pg_sim *sim, pg_object *objects, int32_t n_objects,
                     double *phi, pg_solve_info *info);
int pg_get_phi(pg_sim *sim, double *phi);
/* The potential after the work queued so far, read back without waiting:
 * phi (ndof doubles; page-locked host memory lets the copy overlap the next
 * steps) holds it once pg_synchronize returns.  Keep phi untouched until
 * then; alternate buffers to keep several steps' potentials. */
int pg_get_phi_async(pg_sim *sim, double *phi);
int pg_get_rho(pg_sim *sim, double *rho);
int pg_get_capacitance(pg_sim *sim, double *inv_capacitance);  /* [n_obj][n_obj] */

/* create_flux (punc/src/injector.cpp:104-171) for Maxwellian species. */
int pg_create_flux(pg_sim *sim, const pg_species *species, int32_t n_species);
/* inject_particles (punc/include/punc/injector.h:157-232) with a counter-based
 * Philox4x32-10 stream keyed by (seed, step, species, facet). */
int pg_inject(pg_sim *sim, double dt, uint64_t seed, uint64_t step, int64_t *n_injected);

/* One fused timestep: push, move, update, inject, deposit, Poisson with the
 * circuit, E field (interaction/interaction.cpp:342-480). */
int pg_step(pg_sim *sim, const pg_step_args *args, pg_object *objects, int32_t n_objects,
            pg_step_result *result);
/* n_steps fused timesteps, as n_steps calls of pg_step (same operations and
 * arithmetic; args->step is the first step's RNG counter, incremented per
 * step; args->first_step applies to the first of them), with the particle
 * counts, object charges, currents and potentials and the CircuitCM post-solve
 * kept on the device: no host synchronisation until the end.  use_graph = 1
 * captures a step as a CUDA graph once (per particle buffer and arguments)
 * and replays it.  Cell sorts every sort_interval steps run in between.
 * results (optional): [n_steps]. */
int pg_run_steps(pg_sim *sim, const pg_step_args *args, pg_object *objects, int32_t n_objects,
                 int32_t n_steps, int32_t use_graph, pg_step_result *results);
/* Launch configuration of the particle pass and the cell-sort interval. */
typedef struct pg_tuning {
    int32_t threads;          /* block size of the fused particle pass (0: 256; 32..512) */
    int32_t blocks_per_sm;    /* blocks of the particle pass per SM (0: keep; at most 32) */
    int32_t dep_agg;          /* 1: warp-aggregated fixed-point deposit (mixed form) */
    int32_t sort_interval;    /* steps between cell sorts (0: keep) */
    double pass_ms;           /* autotune: device time of the chosen particle pass */
    double sort_ms;           /* autotune: device time of one cell sort */
} pg_tuning;
int pg_set_tuning(pg_sim *sim, const pg_tuning *tuning);
int pg_get_tuning(pg_sim *sim, pg_tuning *tuning);
/* Autotuner: runs real steps of this simulation (pg_step with args, the RNG
 * step advancing), steps_per_trial for each block size in {128, 256, 512},
 * blocks per SM in {2, 4, 8, 16} and (mixed form) deposit aggregation off/on,
 * keeps the fastest particle pass, then measures one cell sort and the growth
 * of the pass time over 40 steps without sorting and picks the sort interval in
 * {5, 10, 20, 40} of least modelled cost (sort / I + mean growth over I).
 * Applies and returns the choice; about 24 steps_per_trial + 41 steps. */
int pg_autotune(pg_sim *sim, const pg_step_args *args, pg_object *objects, int32_t n_objects,
                int32_t steps_per_trial, pg_tuning *out);
/* Strength threshold theta of the AMG preconditioner's aggregation (the
 * couplings |a_ij| >= theta sqrt(a_ii a_jj) count as strong; 0, the default:
 * every coupling): rebuilds the hierarchy from the matrix kept at pg_create.
 * The solves still stop on the same FP64 residual test; the threshold changes
 * the iteration count and the cost of an iteration.  PG_ERR_ARG without an
 * AMG preconditioner (pcg_precond 1); on failure the previous hierarchy is
 * kept. */
int pg_amg_set_strength(pg_sim *sim, double theta);
int pg_amg_get_strength(pg_sim *sim, double *theta);
/* The threshold chosen by timing: for each candidate (NULL, 0: {0, 0.01,
 * 0.02}) the hierarchy is rebuilt and steps_per_trial real steps of this
 * simulation run (pg_step with args, the RNG step advancing); the candidate
 * of least mean PCG time per step is applied and returned with that time. */
int pg_autotune_amg(pg_sim *sim, const pg_step_args *args, pg_object *objects, int32_t n_objects,
                    int32_t steps_per_trial, const double *thetas, int32_t n_thetas, double *best_theta,
                    double *best_pcg_ms);
/* Adjoint of n_steps fused steps (FP64 form; DG0 field with B = 0, no
 * injection, no absorption, objects at fixed potentials): the forward runs the
 * steps from the current state (args as pg_step; args->step the first step's
 * RNG counter) keeping the particle state every ckpt_every steps, and returns
 * loss = ||rho_K - rho_target||^2 with rho_K the CG1 charge after the steps.
 * Cell sorting is suspended until pg_adjoint_release. */
int pg_adjoint_forward(pg_sim *sim, const pg_step_args *args, pg_object *objects, int32_t n_objects,
                       int32_t n_steps, int32_t ckpt_every, const double *rho_target, double *loss);
/* Gradients of that loss, with each particle's cells fixed from the forward
 * pass (the map is smooth between cell crossings): grad_v [n_out][3] with
 * respect to the initial velocities and grad_x0 [n_out][3] to the initial
 * positions, both indexed by particle id, and grad_E0 [3] to the uniform
 * external field.  Segments between checkpoints are recomputed; the Poisson
 * adjoint is a second PCG on the same symmetric matrix.  Any output may be
 * NULL.  The state returns to the one after the forward steps. */
int pg_adjoint_backward(pg_sim *sim, double *grad_v, int64_t n_out, double *grad_E0, double *grad_x0);
/* After pg_adjoint_backward: the gradient of the loss with respect to the
 * fixed potentials of the objects passed to pg_adjoint_forward (the object
 * bias), grad_pot[k] for object k: phi is affine in each potential V_k with
 * slope the unit-potential Laplace solution L_k, so the gradient is the sum
 * over the steps of <phibar_n, L_k>.  n_objects must match the forward call. */
int pg_adjoint_potential_gradient(pg_sim *sim, double *grad_pot, int32_t n_objects);
int pg_adjoint_release(pg_sim *sim);
/* Sort particles by cell and drop absorbed slots. */
int pg_sort(pg_sim *sim);

/* Per-stage device times in ms of pg_step accumulated since the last call
 * (CUDA events on the engine stream, recorded while profiling is on), like
 * the reference Timer (punc/include/punc/diagnostics.h:171-234). */
int pg_stage_times(pg_sim *sim, double *ms, int32_t capacity, int32_t *n_stages);
const char *pg_stage_name(pg_sim *sim, int32_t index);   /* NULL if out of range */
int pg_set_profiling(pg_sim *sim, int32_t on);
/* CUDA events on the engine stream, for timing a span of calls on the device:
 * record into slot 0..15, then the elapsed ms between two recorded slots
 * (waits for the later one). */
int pg_event_record(pg_sim *sim, int32_t slot);
int pg_event_elapsed(pg_sim *sim, int32_t from_slot, int32_t to_slot, double *ms);
/* Wait until all work queued on the engine stream, and every read-back of
 * pg_get_phi_async, has finished. */
int pg_synchronize(pg_sim *sim);
/* ESolver::solve (punc/src/efield.cpp:70-75, punc/ufl/EField3D.ufl): the CG1
 * field E = L2 projection of -grad(phi) (phi: the current potential), solved
 * by CG on the consistent mass matrix for the three components; FP64 form to
 * rel 1e-12 / abs 1e-14 (the ESolver's tolerances, efield.cpp:62-64), mixed
 * form in FP32 to rel 1e-6.  E (optional): [Ndof][3] on return. */
int pg_esolver_solve(pg_sim *sim, double *E, pg_solve_info *info);
int pg_set_efield_cg1(pg_sim *sim, const double *E);   /* [Ndof][3] */
int pg_get_efield_cg1(pg_sim *sim, double *E);         /* [Ndof][3] */
/* accel_cg1 / boris_cg1 (punc/include/punc/pusher.h:154-201, 282-372): the
 * push with the CG1 field interpolated at each particle; returns KE as
 * pg_accel / pg_boris. */
int pg_accel_cg1(pg_sim *sim, double dt, double *KE);
int pg_boris_cg1(pg_sim *sim, const double B[3], double dt, double *KE);

/* Diagnostics (punc/include/punc/diagnostics.h), on the device particles;
 * species are told apart by the sign of q, as in the reference.
 * particle_potential_energy_cg1 (diagnostics.h:379-412) with the current phi. */
int pg_potential_energy(pg_sim *sim, double *PE);
/* density_cg1 (diagnostics.h:492-555): ne, ni [Ndof], weights w_e, w_i. */
int pg_density_cg1(pg_sim *sim, double weight_e, double weight_i, double *ne, double *ni);
/* density_dg0 (diagnostics.h:433-465): ne, ni [Nc]. */
int pg_density_dg0(pg_sim *sim, double weight_e, double weight_i, double *ne, double *ni);
/* Population::statistics (population.h:746-805): mean speed and sample
 * standard deviation of the negative particles, then of the positive ones
 * (two-pass sums on the device; 0, 0 for a sign without particles). */
int pg_statistics(pg_sim *sim, double *stats);

/* Number of kernels this library has launched in this process. */
int pg_launch_count(int64_t *n);

/* Storage of the Poisson operator and its AMG hierarchy, for diagnostics and
 * traffic models.  The reference's counterpart is PETSc's matrix and hypre's
 * hierarchy statistics (-ksp_view). */
#define PG_MAX_AMG_LEVELS 12
typedef struct pg_poisson_layout {
    int64_t n_rows;                          /* rows of the reduced operator (= dofs) */
    int64_t nnz;                             /* stored nonzeros (exact zeros of K dropped) */
    int64_t sell_entries;                    /* SELL-32 entries including padding */
    int32_t precond;                         /* pg_config.pcg_precond */
    int32_t levels;                          /* AMG levels (0 for Jacobi) */
    int64_t level_rows[PG_MAX_AMG_LEVELS];
    int64_t level_nnz[PG_MAX_AMG_LEVELS];    /* operator nonzeros per level */
    int64_t level_nnz_p[PG_MAX_AMG_LEVELS];  /* nonzeros of the transfer operator S = (I - w D^-1 A) P
                                                to the next level (0 on the coarsest level) */
    int64_t cycle_nnz_g;                     /* entries of G = C^-1 S^T (last restriction + coarse solve) */
    int64_t cycle_nnz_u1;                    /* entries of the collapsed up-sweep operator of levels >= 1 */
    int64_t cycle_bytes;                     /* operator bytes one AMG-PCG iteration reads: stored entries
                                                (padding excluded) times their stored size, each operator
                                                counted once per use */
} pg_poisson_layout;
int pg_poisson_layout_get(pg_sim *sim, pg_poisson_layout *out);

/* Jacobi-preconditioned CG on a caller's CSR matrix (SPD, int32 indices, all
 * arrays in device memory), for callers that cannot allocate device memory:
 * the work vectors live in a static device array of the library instead of
 * buffers from cudaMalloc, and the call allocates nothing.  No counterpart in
 * the reference (it solves through PETSc).  x holds the initial guess and
 * receives the solution; stops when ||b - A x|| <= max(rtol ||b||, atol).
 * At most 524,288 rows (larger n: PG_ERR_ARG); the array (about 20 MB) stays
 * on every GPU that loads the library.  All calls share it, so calls that
 * overlap on the GPU race.  The first call on a device also looks up the
 * array's device address.  stream: a cudaStream_t, or NULL for the default
 * stream; the call waits for the solve to finish. */
int pg_pcg_solve_noalloc(int32_t n, const int32_t *rowptr, const int32_t *col, const double *val,
                         const double *b, double *x, double rtol, double atol, int32_t max_iter,
                         void *stream, int32_t *iterations, double *residual);

#ifdef __cplusplus
}
#endif

#endif /* PUNC_GPU_H */
