// Shifted-Maxwellian flux injection through the exterior facets
// (inject_particles, punc/include/punc/injector.h:157-232).
//
// One thread per (species, exterior facet) owns the Philox stream
// (key = seed, counter words = facet, species, step).  Draw order in a stream:
//   1. one uniform for the Bernoulli rounding of the expected count N,
//   2. for each particle: r, then sqrt(u), placing it on the triangle
//      (random_facet_points, punc/src/injector.cpp:78-102),
//   3. for each particle: rejection sampling of the flux density
//      max(v.n,0) f(v) over the box vd +- vdf_range*vth, 3 uniforms for the
//      candidate and 1 for the test (punc/src/injector.cpp:51-76),
//   4. for each particle: one uniform r, x += r*dt*v.
// The particle is kept if the facet walk from the facet's cell stays inside
// the mesh.  Built with --fmad=false; exp is the portable series so the
// accept/reject decisions equal a CPU evaluation.
#include <cuda_runtime.h>

#include "pg_device.cuh"
#include "pg_math.h"

namespace pg {

namespace {

constexpr int kThreads = 128;
constexpr int kMaxRejections = 1 << 22;

__device__ __forceinline__ void raise_error(DevState *st, int code, int64_t idx) {
    if (atomicCAS(&st->err_code, 0, code) == 0) st->err_index = idx;
}

__device__ __forceinline__ int walk_fp64(const DevMesh &m, double x, double y, double z, int c, int max_steps) {
    for (int it = 0; it < max_steps; ++it) {
        const double2 *P = reinterpret_cast<const double2 *>(m.planes) + 8 * (size_t)c;
        const double2 q0 = __ldg(P + 0), q1 = __ldg(P + 1), q2 = __ldg(P + 2), q3 = __ldg(P + 3);
        const double2 q4 = __ldg(P + 4), q5 = __ldg(P + 5), q6 = __ldg(P + 6), q7 = __ldg(P + 7);
        const int4 nb = __ldg(m.nbr + c);
        double d0 = q0.x + q0.y * x; d0 = d0 + q1.x * y; d0 = d0 + q1.y * z;
        double d1 = q2.x + q2.y * x; d1 = d1 + q3.x * y; d1 = d1 + q3.y * z;
        double d2 = q4.x + q4.y * x; d2 = d2 + q5.x * y; d2 = d2 + q5.y * z;
        double d3 = q6.x + q6.y * x; d3 = d3 + q7.x * y; d3 = d3 + q7.y * z;
        int next;
        if (d0 > 0) next = nb.x;
        else if (d1 > 0) next = nb.y;
        else if (d2 > 0) next = nb.z;
        else if (d3 > 0) next = nb.w;
        else return c;
        if (next < 0) return next;
        c = next;
    }
    return kWalkFail;
}

// Expected count of one stream, rounded by a Bernoulli draw.
__device__ __forceinline__ int64_t stream_count(const InjectParams &ip, const double *flux_num, int idx,
                                                Stream &rs) {
    const int s = idx / ip.n_facets, j = idx % ip.n_facets;
    const double nf = flux_num[idx] * ip.sp[s].ndt;
    int64_t n = (int64_t)nf;
    rs.init(ip.seed, (uint32_t)j, (uint32_t)s, ip.step);
    if (rs.next() < nf - (double)n) n += 1;
    return n;
}

__global__ void k_inject_count(InjectParams ip, const double *__restrict__ flux_num, int64_t *__restrict__ counts) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ip.n_species * ip.n_facets) return;
    Stream rs;
    counts[idx] = stream_count(ip, flux_num, idx, rs);
}

__global__ void k_inject_generate(DevMesh m, DevParticles p, InjectParams ip, const double *__restrict__ flux_num,
                                  const double *__restrict__ pdf_max, const double *__restrict__ facets,
                                  const int64_t *__restrict__ offsets, int max_steps, int deposit,
                                  const double *__restrict__ qsp, double *__restrict__ rho_acc,
                                  DevState *__restrict__ st) {
    const int total = ip.n_species * ip.n_facets;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    if (idx == total - 1) st->inject_total = offsets[idx] + (offsets[total] - offsets[idx]);
    Stream rs;
    const int64_t n = stream_count(ip, flux_num, idx, rs);
    if (n == 0) return;
    const int s = idx / ip.n_facets, j = idx % ip.n_facets;
    const InjectSpecies &S = ip.sp[s];
    const double *F = facets + 14 * (size_t)j;
    const double v0x = F[1], v0y = F[2], v0z = F[3];
    const double v1x = F[4], v1y = F[5], v1z = F[6];
    const double v2x = F[7], v2y = F[8], v2z = F[9];
    const double nx = F[10], ny = F[11], nz = F[12];
    const int cell0 = (int)F[13];
    const int64_t base = ip.slot_base + offsets[idx];
    // 2. positions on the triangle
    for (int64_t k = 0; k < n; ++k) {
        const double r = rs.next();
        double x = (1.0 - r) * v0x + r * v1x;
        double y = (1.0 - r) * v0y + r * v1y;
        double z = (1.0 - r) * v0z + r * v1z;
        const double r2 = sqrt(rs.next());
        x = r2 * x + (1.0 - r2) * v2x;
        y = r2 * y + (1.0 - r2) * v2y;
        z = r2 * z + (1.0 - r2) * v2z;
        p.x[base + k] = x; p.y[base + k] = y; p.z[base + k] = z;
    }
    // 3. velocities from the flux density
    const double pmax = pdf_max[idx];
    for (int64_t k = 0; k < n; ++k) {
        double tx = 0, ty = 0, tz = 0;
        int tries = 0;
        for (;;) {
            tx = S.domain_lo[0] + S.domain_w[0] * rs.next();
            ty = S.domain_lo[1] + S.domain_w[1] * rs.next();
            tz = S.domain_lo[2] + S.domain_w[2] * rs.next();
            const double u = rs.next();
            double vn = 0.0;
            vn += tx * nx; vn += ty * ny; vn += tz * nz;
            double vs = 0.0;
            vs += (tx - S.vd[0]) * (tx - S.vd[0]);
            vs += (ty - S.vd[1]) * (ty - S.vd[1]);
            vs += (tz - S.vd[2]) * (tz - S.vd[2]);
            const double f = S.factor * exp_portable(-0.5 * vs / S.vth2);
            const double pdf = (double)(vn > 0.0) * vn * f;
            if (u * pmax < pdf) break;
            if (++tries >= kMaxRejections) { raise_error(st, PG_ERR_ARG, idx); return; }
        }
        p.vx[base + k] = tx; p.vy[base + k] = ty; p.vz[base + k] = tz;
    }
    // 4. advance into the domain and locate by walking from the facet's cell
    int64_t kept = 0;
    for (int64_t k = 0; k < n; ++k) {
        const double r = rs.next();
        const int64_t i = base + k;
        const double vx = p.vx[i], vy = p.vy[i], vz = p.vz[i];
        const double x = p.x[i] + r * ip.dt * vx;
        const double y = p.y[i] + r * ip.dt * vy;
        const double z = p.z[i] + r * ip.dt * vz;
        p.x[i] = x; p.y[i] = y; p.z[i] = z;
        p.sp[i] = (uint8_t)s;
        p.pid[i] = ip.pid_base + offsets[idx] + k;
        const int c = walk_fp64(m, x, y, z, cell0, max_steps);
        if (c == kWalkFail) { raise_error(st, PG_ERR_WALK_LIMIT, i); p.cell[i] = kDead; continue; }
        if (c < 0) { p.cell[i] = kDead; continue; }
        p.cell[i] = c;
        ++kept;
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
    if (kept) {
        atomicAdd(reinterpret_cast<unsigned long long *>(&st->injected[s]), (unsigned long long)kept);
        atomicAdd(reinterpret_cast<unsigned long long *>(&st->live[s]), (unsigned long long)kept);
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
                            cudaStream_t st) {
    const int total = ip.n_species * ip.n_facets;
    if (total <= 0) return;
    count_launches(1);
    k_inject_generate<<<(total + kThreads - 1) / kThreads, kThreads, 0, st>>>(
        m, p, ip, flux_num, pdf_max, facets, offsets, max_steps, deposit, q_species, rho_acc, state);
}

}  // namespace pg
