// Species weights of the C++ front end (include/punc_gpu.hpp make_species,
// min_plasma_period) on a mesh read from raw arrays; prints one line per
// amount type: weight q m n num debye, then the plasma period and the mesh
// volume, then the sums of element_volume with and without voronoi, all %.17g.
// Host only: building the mesh tables needs no GPU.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "punc_gpu.hpp"

template <class T>
static std::vector<T> read_all(const char *path) {
    std::vector<T> v;
    FILE *f = std::fopen(path, "rb");
    if (!f) return v;
    T x;
    while (std::fread(&x, sizeof(T), 1, f) == 1) v.push_back(x);
    std::fclose(f);
    return v;
}

// Compiled, not run (it needs a GPU): the Particle<3> overload of
// add_particles type-checks against the reference's record.
[[maybe_unused]] static void add_records(punc::gpu::Population<3> &pop) {
    const double x[3] = {0.1, 0.2, 0.3}, v[3] = {1.0, 0.0, 0.0};
    std::vector<punc::gpu::Particle<3>> ps{punc::gpu::Particle<3>(x, v, -1.0, 1.0), punc::gpu::Particle<3>()};
    static_assert(sizeof(punc::gpu::Particle<3>) == 64, "64-byte particle record");
    pop.add_particles(ps);
}

int main(int argc, char **argv) {
    if (argc < 5) return 2;
    const auto coords = read_all<double>(argv[1]);
    const auto cells = read_all<int64_t>(argv[2]);
    const auto bf = read_all<int64_t>(argv[3]);
    const auto bt = read_all<int32_t>(argv[4]);
    punc::gpu::Mesh mesh(coords, cells, bf, bt, 1.0);
    using T = punc::gpu::ParticleAmountType;
    const T types[] = {T::in_total, T::per_cell, T::per_volume, T::phys_per_sim};
    const double amounts[] = {20000.0, 16.0, 40.0, 3.0};
    const double vd[3] = {0.5, 0.0, -0.25};
    std::vector<punc::gpu::Species> all;
    for (int k = 0; k < 4; ++k) {
        const auto s = punc::gpu::make_species(-1.0, 1.0, 100.0, amounts[k], types[k], mesh, 1.0, vd);
        std::printf("%.17g %.17g %.17g %.17g %zu %.17g\n", s.weight, s.q, s.m, s.n, s.num, s.debye);
        all.push_back(s);
        all.push_back(punc::gpu::make_species(1.0, 1836.0, 100.0, amounts[k], types[k], mesh, 0.05));
    }
    std::printf("%.17g %.17g\n", punc::gpu::min_plasma_period(all, 1.0), mesh.volume());
    const auto dv = punc::gpu::element_volume(mesh, true), dv1 = punc::gpu::element_volume(mesh, false);
    double s_dv = 0.0, s_dv1 = 0.0;
    for (std::size_t k = 0; k < dv.size(); ++k) { s_dv += dv[k]; s_dv1 += dv1[k]; }
    std::printf("%.17g %.17g\n", s_dv, s_dv1);
    return 0;
}
