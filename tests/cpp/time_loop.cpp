// A PUNC++-shaped time loop (interaction/interaction.cpp:342-480) against the
// C++ front end of the engine; compiled and linked by tests/test_abi.py.
#include <cstdio>
#include <vector>

#include "punc_gpu.hpp"

namespace pg = punc::gpu;

int main() {
    // one unit cube split into 6 tetrahedra, all 12 boundary facets exterior
    std::vector<double> coords;
    for (int i = 0; i < 8; ++i) { coords.push_back(i & 1); coords.push_back((i >> 1) & 1); coords.push_back((i >> 2) & 1); }
    std::vector<int64_t> cells = {0, 1, 3, 7, 0, 1, 5, 7, 0, 2, 3, 7, 0, 2, 6, 7, 0, 4, 5, 7, 0, 4, 6, 7};
    std::vector<int64_t> bf = {0, 1, 3, 0, 2, 3, 4, 5, 7, 4, 6, 7, 0, 1, 5, 0, 4, 5, 2, 3, 7, 2, 6, 7,
                               0, 2, 6, 0, 4, 6, 1, 3, 7, 1, 5, 7};
    std::vector<int32_t> tags(12, 1);
    pg::Mesh mesh(coords, cells, bf, tags);
    pg::Population<3> pop(mesh);
    pop.add_particles({0.5, 0.5, 0.5}, {0.1, 0.0, 0.0}, -1.0, 1.0);
    pg::Function rho(pop, pg::Function::Rho), phi(pop, pg::Function::Phi), E(pop, pg::Function::E);
    pg::ObjectVector objects;
    pg::PoissonSolver poisson(pop);
    pg::EFieldDG0 esolver;
    std::vector<double> B = {0, 0, 0}, dv_inv;
    const double dt = 0.1;
    for (int n = 0; n < 3; ++n) {
        pg::distribute_cg1(pop, rho, dv_inv);
        poisson.solve(phi, rho, objects);
        esolver.solve(E, phi);
        double KE = pg::boris(pop, E, B, (1.0 - 0.5 * (n == 0)) * dt);
        pg::move(pop, dt);
        pop.update(objects, dt);
        std::printf("step %d KE %.6e particles %zu\n", n, KE, pop.num_of_particles());
    }
    // the same loop body as fused steps replayed from a captured graph
    pg_step_args args{};
    args.dt = dt;
    args.step = 3;
    for (const pg_step_result &r : pg::run_steps(pop, objects, args, 2, true))
        std::printf("fused KE %.6e particles %lld\n", r.KE, (long long)r.n_particles);
    return 0;
}
