// On-device diagnostics of the reference (punc/include/punc/diagnostics.h,
// punc/include/punc/population.h:746-805), both particle forms:
//   particle_potential_energy_cg1  PE = sum_p 0.5 q_p phi(x_p)
//   density_cg1                    n_s,j = dv_inv_j w_s sum_{p in s} lambda_j(x_p)
//   density_dg0                    n_s,T = (count of s in T) w_s / vol_T
//   Population::statistics         mean and standard deviation of the speed of
//                                  the negative and the positive particles
// Species are told apart by the sign of q, as in the reference.  Sums are
// parallel reductions or FP64 atomics (order-dependent last bits); the
// statistics use two passes (mean, then squared deviations) in place of the
// reference's sequential Welford recurrence (same quantities).
#include <cuda_runtime.h>

#include "pg_device.cuh"
#include "pg_walk.cuh"

namespace pg {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ void block_add(double v, double *sh, double *out) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        double s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) atomicAdd(out, s);
    }
    __syncthreads();
}

// position and barycentric weights of slot i (FP64 or FP32 form)
template <bool MIXED>
__device__ __forceinline__ void lambdas(const DevMesh &m, const DevParticles &p, int64_t i, int c, double &l0,
                                        double &l1, double &l2, double &l3) {
    if (MIXED) {
        const float x = p.xf[i], y = p.yf[i], z = p.zf[i];
        const float4 *A = m.cell_f + 4 * (size_t)c;
        const float4 a0 = __ldg(A), a1 = __ldg(A + 1), a2 = __ldg(A + 2);
        const float f0 = fmaf(a0.w, z, fmaf(a0.z, y, fmaf(a0.y, x, a0.x)));
        const float f1 = fmaf(a1.w, z, fmaf(a1.z, y, fmaf(a1.y, x, a1.x)));
        const float f2 = fmaf(a2.w, z, fmaf(a2.z, y, fmaf(a2.y, x, a2.x)));
        l0 = f0; l1 = f1; l2 = f2; l3 = (double)(1.0f - f0 - f1 - f2);
    } else {
        barycentric_fp64(m, c, p.x[i], p.y[i], p.z[i], l0, l1, l2, l3);
    }
}

template <bool MIXED>
__device__ __forceinline__ double speed(const DevParticles &p, int64_t i) {
    double v = 0.0;
    if (MIXED) {
        const double a = p.vxf[i], b = p.vyf[i], c = p.vzf[i];
        v += a * a; v += b * b; v += c * c;
    } else {
        v += p.vx[i] * p.vx[i]; v += p.vy[i] * p.vy[i]; v += p.vz[i] * p.vz[i];
    }
    return sqrt(v);
}

// particle_potential_energy_cg1 (punc/include/punc/diagnostics.h:379-412):
// phi_x = sum_i coeffs[i] * values[i]; PE += 0.5 * q * phi_x.
template <bool MIXED>
__global__ void k_potential_energy(DevMesh m, DevParticles p, int64_t n_slots, const double *__restrict__ qsp,
                                   const double *__restrict__ phi, double *__restrict__ out) {
    __shared__ double sh[32];
    double pe = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_slots; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = p.cell[i];
        if (c < 0) continue;
        double l0, l1, l2, l3;
        lambdas<MIXED>(m, p, i, c, l0, l1, l2, l3);
        const int4 d = __ldg(m.dofs + c);
        double phx = l0 * phi[d.x];
        phx = phx + l1 * phi[d.y];
        phx = phx + l2 * phi[d.z];
        phx = phx + l3 * phi[d.w];
        pe += 0.5 * qsp[p.sp[i]] * phx;
    }
    block_add(pe, sh, out);
}

// density_cg1 (punc/include/punc/diagnostics.h:492-555): sum of lambda_j per sign.
template <bool MIXED>
__global__ void k_density_cg1(DevMesh m, DevParticles p, int64_t n_slots, const double *__restrict__ qsp,
                              double *__restrict__ acc_e, double *__restrict__ acc_i) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_slots; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = p.cell[i];
        if (c < 0) continue;
        double l0, l1, l2, l3;
        lambdas<MIXED>(m, p, i, c, l0, l1, l2, l3);
        const double q = qsp[p.sp[i]];
        if (q == 0.0) continue;
        double *acc = q < 0.0 ? acc_e : acc_i;
        const int4 d = __ldg(m.dofs + c);
        atomicAdd(acc + d.x, l0);
        atomicAdd(acc + d.y, l1);
        atomicAdd(acc + d.z, l2);
        atomicAdd(acc + d.w, l3);
    }
}

__global__ void k_density_cg1_finish(int32_t n, const double *__restrict__ dv_inv, double we, double wi,
                                     double *__restrict__ ne, double *__restrict__ ni) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    ne[i] = ne[i] * (dv_inv[i] * we);
    ni[i] = ni[i] * (dv_inv[i] * wi);
}

// density_dg0 (punc/include/punc/diagnostics.h:433-465): particle counts per cell and sign.
__global__ void k_density_dg0(DevParticles p, int64_t n_slots, const double *__restrict__ qsp,
                              unsigned long long *__restrict__ cnt) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_slots; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = p.cell[i];
        if (c < 0) continue;
        const double q = qsp[p.sp[i]];
        if (q == 0.0) continue;
        atomicAdd(cnt + 2 * (size_t)c + (q < 0.0 ? 0 : 1), 1ull);
    }
}

__global__ void k_density_dg0_finish(int32_t nc, const unsigned long long *__restrict__ cnt,
                                     const double *__restrict__ vol, double we, double wi, double *__restrict__ ne,
                                     double *__restrict__ ni) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    ne[c] = ((double)cnt[2 * (size_t)c] * we) / vol[c];
    ni[c] = ((double)cnt[2 * (size_t)c + 1] * wi) / vol[c];
}

// Population::statistics (punc/include/punc/population.h:746-805), pass 1:
// counts and speed sums per sign; pass 2: squared deviations from the means.
template <bool MIXED>
__global__ void k_stats(DevParticles p, int64_t n_slots, const double *__restrict__ qsp, int pass,
                        double *__restrict__ acc) {
    __shared__ double sh[32];
    double ne = 0.0, ni = 0.0, se = 0.0, si = 0.0;
    const double me = pass ? acc[1] / fmax(acc[0], 1.0) : 0.0, mi = pass ? acc[3] / fmax(acc[2], 1.0) : 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_slots; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = p.cell[i];
        if (c < 0) continue;
        const double q = qsp[p.sp[i]];
        const double v = speed<MIXED>(p, i);
        if (q < 0.0) {
            if (pass) { const double d = v - me; se += d * d; } else { ne += 1.0; se += v; }
        } else if (q > 0.0) {
            if (pass) { const double d = v - mi; si += d * d; } else { ni += 1.0; si += v; }
        }
    }
    if (pass) {
        block_add(se, sh, acc + 4);
        block_add(si, sh, acc + 5);
    } else {
        block_add(ne, sh, acc + 0);
        block_add(se, sh, acc + 1);
        block_add(ni, sh, acc + 2);
        block_add(si, sh, acc + 3);
    }
}

int blocks_for(int64_t n) {
    int64_t g = (n + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)sm_count() * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

void launch_potential_energy(const DevMesh &m, const DevParticles &p, int64_t n_slots, bool mixed,
                             const double *qsp, const double *phi, double *out, cudaStream_t st) {
    cudaMemsetAsync(out, 0, sizeof(double), st);
    if (n_slots <= 0) return;
    count_launches(1);
    if (mixed) k_potential_energy<true><<<blocks_for(n_slots), kThreads, 0, st>>>(m, p, n_slots, qsp, phi, out);
    else k_potential_energy<false><<<blocks_for(n_slots), kThreads, 0, st>>>(m, p, n_slots, qsp, phi, out);
}

void launch_density_cg1(const DevMesh &m, const DevParticles &p, int64_t n_slots, bool mixed, const double *qsp,
                        double we, double wi, double *ne, double *ni, cudaStream_t st) {
    cudaMemsetAsync(ne, 0, sizeof(double) * m.ndof, st);
    cudaMemsetAsync(ni, 0, sizeof(double) * m.ndof, st);
    count_launches(2);
    if (n_slots > 0) {
        if (mixed) k_density_cg1<true><<<blocks_for(n_slots), kThreads, 0, st>>>(m, p, n_slots, qsp, ne, ni);
        else k_density_cg1<false><<<blocks_for(n_slots), kThreads, 0, st>>>(m, p, n_slots, qsp, ne, ni);
    }
    k_density_cg1_finish<<<(m.ndof + kThreads - 1) / kThreads, kThreads, 0, st>>>(m.ndof, m.dv_inv, we, wi, ne, ni);
}

void launch_density_dg0(const DevMesh &m, const DevParticles &p, int64_t n_slots, const double *qsp,
                        const double *vol, double we, double wi, unsigned long long *cnt, double *ne, double *ni,
                        cudaStream_t st) {
    cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * 2 * m.nc, st);
    count_launches(2);
    if (n_slots > 0) k_density_dg0<<<blocks_for(n_slots), kThreads, 0, st>>>(p, n_slots, qsp, cnt);
    k_density_dg0_finish<<<(m.nc + kThreads - 1) / kThreads, kThreads, 0, st>>>(m.nc, cnt, vol, we, wi, ne, ni);
}

void launch_statistics(const DevParticles &p, int64_t n_slots, bool mixed, const double *qsp, double *acc,
                       cudaStream_t st) {
    cudaMemsetAsync(acc, 0, sizeof(double) * 6, st);
    if (n_slots <= 0) return;
    count_launches(2);
    for (int pass = 0; pass < 2; ++pass) {
        if (mixed) k_stats<true><<<blocks_for(n_slots), kThreads, 0, st>>>(p, n_slots, qsp, pass, acc);
        else k_stats<false><<<blocks_for(n_slots), kThreads, 0, st>>>(p, n_slots, qsp, pass, acc);
    }
}

}  // namespace pg
