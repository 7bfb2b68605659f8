// Shifted-Maxwellian flux injection through the exterior facets
// (inject_particles, punc/include/punc/injector.h:157-232).
//
// Random numbers come from Philox4x32-10 with key = seed and counter words
// (block, c1, c2, c3); each block gives two uniforms.
//   count stream of (species s, facet j):  c1 = j, c2 = s, c3 = step;
//     block 0, first uniform: Bernoulli rounding of the expected count
//     N = flux * n * dt (punc/include/punc/injector.h:183-191).
//   stream of particle k of (s, j):         c1 = j, c2 = s + 8 (k + 1), c3 = step;
//     block 0: r1, r2 -> uniform point on the facet triangle
//              (random_facet_points, punc/src/injector.cpp:78-102);
//     block 1: r  -> the particle is advanced by r dt v (injector.h:209-217);
//     blocks 2+2i, 3+2i: candidate i of the rejection sampler of the flux
//              density max(v.n, 0) f(v) over vd +- vdf_range vth
//              (punc/src/injector.cpp:51-76): three uniforms for v, one for the
//              test; the first accepted candidate is kept.
// Because every candidate has its own counter, a warp tests 32 candidates of
// one particle at once and keeps the lowest accepted index, which is exactly
// the sequential loop's choice.  The particle is kept if the facet walk from
// the facet's cell stays in the mesh.  Built with --fmad=false; exp is the
// portable series, so accept/reject decisions equal a CPU evaluation.  Each
// candidate is first decided in FP32 with an error bound (pg_screen.h); the
// FP64 test runs only when the FP32 margin is inside the bound.  The FP64 form
// forms the kept particle's velocity and position in FP64 (the oracle's bits);
// the mixed form forms them in FP32 from the same random words (the top 24
// bits of each uniform) and an FP32 copy of the facet.
#include <cuda_runtime.h>

#include <algorithm>

#include "pg_device.cuh"
#include "pg_math.h"
#include "pg_screen.h"
#include "pg_walk.cuh"

namespace pg {

namespace {

constexpr int kThreads = 128;
constexpr int kMaxRounds = 1 << 16;   // 2M candidates per particle before giving up

__device__ __forceinline__ void uniforms2(uint64_t seed, uint32_t block, uint32_t c1, uint32_t c2, uint32_t c3,
                                          double &a, double &b) {
    const Philox4 r = philox4x32_10(block, c1, c2, c3, uint32_t(seed), uint32_t(seed >> 32));
    a = u01_from(r.v[0], r.v[1]);
    b = u01_from(r.v[2], r.v[3]);
}

__global__ void k_inject_count(InjectParams ip, const double *__restrict__ flux_num, int64_t *__restrict__ counts) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ip.n_species * ip.n_facets) return;
    const int s = idx / ip.n_facets, j = idx % ip.n_facets;
    const double nf = flux_num[idx] * ip.sp[s].ndt;
    int64_t n = (int64_t)nf;
    double u, unused;
    const uint32_t step = ip.counts_dev ? (uint32_t)ip.counts_dev[2] : ip.step;
    const uint64_t seed = ip.facet_seed ? ip.seed + ip.facet_seed[j] : ip.seed;
    const uint32_t c1 = ip.facet_c1 ? ip.facet_c1[j] : (uint32_t)j;
    uniforms2(seed, 0u, c1, (uint32_t)s, step, u, unused);
    if (u < nf - (double)n) n += 1;
    counts[idx] = n;
}

// One warp per group of G consecutive injected particles (grid-stride over
// groups; G = the particles per warp of the launch, 1..32, so that small
// injections still spread over every warp): each of lanes 0..G-1 finds its
// particle's stream (a binary search over the stream offsets) and loads what
// the sampling needs, all at once; the warp then samples the group's
// velocities one particle after another (32 candidates a round, the first
// accepted one kept by the particle's lane); finally each lane forms its
// particle's position, walks it from the facet's cell and deposits it. The
// arithmetic of every particle is the one-particle-at-a-time sequence.
__global__ void __launch_bounds__(kThreads, 8) k_inject_generate(DevMesh m, DevParticles p, InjectParams ip, const double *__restrict__ pdf_max,
                                  const double *__restrict__ facets, const int64_t *__restrict__ offsets,
                                  int max_steps, int deposit, const double *__restrict__ qsp,
                                  double *__restrict__ rho_acc, DevState *__restrict__ st) {
    const int total_streams = ip.n_species * ip.n_facets;
    const int64_t total = offsets[total_streams];
    const int64_t slot_base = ip.counts_dev ? ip.counts_dev[0] : ip.slot_base;
    const int64_t pid_base = ip.counts_dev ? ip.counts_dev[1] : ip.pid_base;
    const uint32_t step = ip.counts_dev ? (uint32_t)ip.counts_dev[2] : ip.step;
    const bool mixed = p.xf != nullptr;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    if (warp == 0 && lane == 0) st->inject_total = total;
    const int64_t per_warp = (total + nwarps - 1) / nwarps;
    const int G = per_warp < 1 ? 1 : per_warp > 32 ? 32 : (int)per_warp;
    for (int64_t g0 = warp * G; g0 < total; g0 += nwarps * G) {
        // this lane's particle t and its stream idx: the last idx with
        // offsets[idx] <= t
        const int64_t t = g0 + lane;
        const bool mine = lane < G && t < total;
        int idx = 0;
        if (mine) {
            int lo = 0, hi = total_streams;
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (offsets[mid] <= t) lo = mid; else hi = mid;
            }
            idx = lo;
        }
        const int64_t k = mine ? t - offsets[idx] : 0;
        const int s = idx / ip.n_facets, j = idx % ip.n_facets;
        const double *F = facets + 14 * (size_t)j;
        const uint32_t c1 = ip.facet_c1 ? ip.facet_c1[j] : (uint32_t)j, c2 = (uint32_t)(s + 8 * (k + 1));
        const uint64_t seed = ip.facet_seed ? ip.seed + ip.facet_seed[j] : ip.seed;
        const double pmax = mine ? pdf_max[idx] : 0.0;
        double nx = 0.0, ny = 0.0, nz = 0.0;
        float nx32, ny32, nz32;
        if (mixed) {
            const float4 G2 = __ldg(ip.facets_f + 4 * (size_t)j + 2);
            nx32 = G2.y; ny32 = G2.z; nz32 = G2.w;
        }
        if (mine) { nx = F[10]; ny = F[11]; nz = F[12]; }
        if (!mixed) { nx32 = (float)nx; ny32 = (float)ny; nz32 = (float)nz; }
        // rejection sampling of the group's particles in turn; each candidate
        // is screened in FP32 and only undecided ones take the FP64 test
        uint32_t wv0 = 0, wv1 = 0, wv2 = 0, wv3 = 0, wv4 = 0, wv5 = 0;   // this lane's accepted candidate
        int found = -1;
        const int n_group = total - g0 < G ? (int)(total - g0) : G;
        for (int q = 0; q < n_group; ++q) {
            const int sq = __shfl_sync(0xffffffffu, s, q);
            const uint32_t qc1 = __shfl_sync(0xffffffffu, c1, q), qc2 = __shfl_sync(0xffffffffu, c2, q);
            const uint64_t qseed = __shfl_sync(0xffffffffu, seed, q);
            const double qpmax = __shfl_sync(0xffffffffu, pmax, q);
            const double qnx = __shfl_sync(0xffffffffu, nx, q), qny = __shfl_sync(0xffffffffu, ny, q);
            const double qnz = __shfl_sync(0xffffffffu, nz, q);
            const float qnx32 = __shfl_sync(0xffffffffu, nx32, q), qny32 = __shfl_sync(0xffffffffu, ny32, q);
            const float qnz32 = __shfl_sync(0xffffffffu, nz32, q);
            const InjectSpecies &S = ip.sp[sq];
            FluxBox B;
            for (int c = 0; c < 3; ++c) { B.lo[c] = S.domain_lo[c]; B.w[c] = S.domain_w[c]; B.vd[c] = S.vd[c]; }
            B.vth2 = S.vth2;
            B.factor = S.factor;
            const FluxBox32 &B32 = ip.sp32[sq];
            const float pmax32 = (float)qpmax;
            const uint32_t k0 = uint32_t(qseed), k1 = uint32_t(qseed >> 32);
            int qfound = -1;
            for (int round = 0; round < kMaxRounds && qfound < 0; ++round) {
                const uint32_t cand = (uint32_t)round * 32u + (uint32_t)lane;
                const Philox4 ra = philox4x32_10(2u + 2u * cand, qc1, qc2, step, k0, k1);
                const Philox4 rb = philox4x32_10(3u + 2u * cand, qc1, qc2, step, k0, k1);
                int dec = flux_screen_fp32(B32, qnx32, qny32, qnz32, pmax32, ra.v[0], ra.v[2], rb.v[0], rb.v[2]);
                if (dec < 0) {
                    double tv[3];
                    dec = flux_accept_fp64(B, qnx, qny, qnz, qpmax, u01_from(ra.v[0], ra.v[1]),
                                           u01_from(ra.v[2], ra.v[3]), u01_from(rb.v[0], rb.v[1]),
                                           u01_from(rb.v[2], rb.v[3]), tv) ? 1 : 0;
                }
                const unsigned acc = __ballot_sync(0xffffffffu, dec == 1);
                if (acc) {
                    const int first = __ffs(acc) - 1;
                    qfound = first;
                    const uint32_t a0 = __shfl_sync(0xffffffffu, ra.v[0], first);
                    const uint32_t a1 = __shfl_sync(0xffffffffu, ra.v[1], first);
                    const uint32_t a2 = __shfl_sync(0xffffffffu, ra.v[2], first);
                    const uint32_t a3 = __shfl_sync(0xffffffffu, ra.v[3], first);
                    const uint32_t a4 = __shfl_sync(0xffffffffu, rb.v[0], first);
                    const uint32_t a5 = __shfl_sync(0xffffffffu, rb.v[1], first);
                    if (lane == q) { found = first; wv0 = a0; wv1 = a1; wv2 = a2; wv3 = a3; wv4 = a4; wv5 = a5; }
                }
            }
        }
        if (!mine) continue;
        const int64_t i = slot_base + t;
        p.sp[i] = (uint8_t)s;
        p.pid[i] = pid_base + t;
        if (found < 0) { raise_device_error(st, PG_ERR_ARG, idx); p.cell[i] = kDead; continue; }
        const uint32_t k0 = uint32_t(seed), k1 = uint32_t(seed >> 32);
        if (mixed) {
            // mixed form: the velocity and the position in FP32 from the same
            // random words (24-bit uniforms), the facet in FP32; the
            // acceptance above is the FP64 decision
            const FluxBox32 &B32 = ip.sp32[s];
            const float4 *G = ip.facets_f + 4 * (size_t)j;
            const float4 G0 = __ldg(G), G1 = __ldg(G + 1), G2 = __ldg(G + 2), G3 = __ldg(G + 3);
            const float vxf = B32.lo[0] + B32.w[0] * u01_24(wv0);
            const float vyf = B32.lo[1] + B32.w[1] * u01_24(wv2);
            const float vzf = B32.lo[2] + B32.w[2] * u01_24(wv4);
            const Philox4 q0 = philox4x32_10(0u, c1, c2, step, k0, k1);
            const Philox4 q1 = philox4x32_10(1u, c1, c2, step, k0, k1);
            const float r1 = u01_24(q0.v[0]), r2 = u01_24(q0.v[2]), r = u01_24(q1.v[0]);
            float x = (1.0f - r1) * G0.x + r1 * G0.w;
            float y = (1.0f - r1) * G0.y + r1 * G1.x;
            float z = (1.0f - r1) * G0.z + r1 * G1.y;
            const float sr = sqrtf(r2);
            x = sr * x + (1.0f - sr) * G1.z;
            y = sr * y + (1.0f - sr) * G1.w;
            z = sr * z + (1.0f - sr) * G2.x;
            const float rdt = r * (float)ip.dt;
            x = x + rdt * vxf;
            y = y + rdt * vyf;
            z = z + rdt * vzf;
            p.xf[i] = x; p.yf[i] = y; p.zf[i] = z;
            p.vxf[i] = vxf; p.vyf[i] = vyf; p.vzf[i] = vzf;
            int retests = 0;
            const int c = walk_mixed(m, x, y, z, __float_as_int(G3.x), max_steps, retests);
            if (c == kWalkFail) { raise_device_error(st, PG_ERR_WALK_LIMIT, i); p.cell[i] = kDead; continue; }
            if (c < 0) { p.cell[i] = kDead; continue; }
            p.cell[i] = c;
            atomicAdd(reinterpret_cast<unsigned long long *>(&st->injected[s]), 1ull);
            atomicAdd(reinterpret_cast<unsigned long long *>(&st->live[s]), 1ull);
            if (deposit) deposit_fixed(m, c, x, y, z, ip.q_scaled[s], ip.rho_fixed);
            continue;
        }
        const InjectSpecies &S = ip.sp[s];
        const double vx = S.domain_lo[0] + S.domain_w[0] * u01_from(wv0, wv1);
        const double vy = S.domain_lo[1] + S.domain_w[1] * u01_from(wv2, wv3);
        const double vz = S.domain_lo[2] + S.domain_w[2] * u01_from(wv4, wv5);
        double r1, r2, r, unused;
        uniforms2(seed, 0u, c1, c2, step, r1, r2);
        uniforms2(seed, 1u, c1, c2, step, r, unused);
        double x = (1.0 - r1) * F[1] + r1 * F[4];
        double y = (1.0 - r1) * F[2] + r1 * F[5];
        double z = (1.0 - r1) * F[3] + r1 * F[6];
        const double sr = sqrt(r2);
        x = sr * x + (1.0 - sr) * F[7];
        y = sr * y + (1.0 - sr) * F[8];
        z = sr * z + (1.0 - sr) * F[9];
        x = x + r * ip.dt * vx;
        y = y + r * ip.dt * vy;
        z = z + r * ip.dt * vz;
        p.x[i] = x; p.y[i] = y; p.z[i] = z;
        p.vx[i] = vx; p.vy[i] = vy; p.vz[i] = vz;
        const int c = walk_fp64(m, x, y, z, (int)F[13], max_steps);
        if (c == kWalkFail) { raise_device_error(st, PG_ERR_WALK_LIMIT, i); p.cell[i] = kDead; continue; }
        if (c < 0) { p.cell[i] = kDead; continue; }
        p.cell[i] = c;
        atomicAdd(reinterpret_cast<unsigned long long *>(&st->injected[s]), 1ull);
        atomicAdd(reinterpret_cast<unsigned long long *>(&st->live[s]), 1ull);
        if (deposit) {
            const double2 *A = reinterpret_cast<const double2 *>(m.bary) + 6 * (size_t)c;
            const double2 a0 = A[0], a1 = A[1], a2 = A[2], a3 = A[3], a4 = A[4], a5 = A[5];
            double l0 = a0.x + a0.y * x; l0 = l0 + a1.x * y; l0 = l0 + a1.y * z;
            double l1 = a2.x + a2.y * x; l1 = l1 + a3.x * y; l1 = l1 + a3.y * z;
            double l2 = a4.x + a4.y * x; l2 = l2 + a5.x * y; l2 = l2 + a5.y * z;
            const double l3 = 1.0 - l0 - l1 - l2;
            const double q = qsp[s];
            const int4 d = m.dofs[c];
            atomicAdd(rho_acc + d.x, q * l0);
            atomicAdd(rho_acc + d.y, q * l1);
            atomicAdd(rho_acc + d.z, q * l2);
            atomicAdd(rho_acc + d.w, q * l3);
        }
    }
}

}  // namespace

void launch_inject_count(const DevMesh &m, const InjectParams &ip, const double *flux_num, int64_t *counts,
                         cudaStream_t st) {
    (void)m;
    const int total = ip.n_species * ip.n_facets;
    if (total <= 0) return;
    count_launches(1);
    k_inject_count<<<(total + kThreads - 1) / kThreads, kThreads, 0, st>>>(ip, flux_num, counts);
}

void launch_inject_generate(const DevMesh &m, const DevParticles &p, const InjectParams &ip, const double *flux_num,
                            const double *pdf_max, const double *facets, const int64_t *offsets, int max_steps,
                            int deposit, const double *q_species, double *rho_acc, DevState *state,
                            int64_t max_particles, cudaStream_t st) {
    (void)flux_num;
    if (ip.n_species * ip.n_facets <= 0) return;
    const int64_t warps = std::max<int64_t>(1, std::min<int64_t>(max_particles, (int64_t)sm_count() * 64));
    const int64_t blocks = (warps * 32 + kThreads - 1) / kThreads;
    count_launches(1);
    k_inject_generate<<<(unsigned)blocks, kThreads, 0, st>>>(m, p, ip, pdf_max, facets, offsets, max_steps, deposit,
                                                             q_species, rho_acc, state);
}

}  // namespace pg
