// Mixed-precision particle kernels: FP32 positions and velocities, the DG0
// field formed from the potential at the particle's cell, FP32 push and move
// with fused multiply-adds, the FP32 facet walk (the sign of each barycentric
// coordinate, with an FP64 re-test of facets the particle lies within the
// FP32 error bound of), and the int64 fixed-point CG1 deposit (bitwise
// identical from run to run) from the walk's last barycentric coordinates.
//
// Per particle a pass reads 24 B of FP32 position and velocity, 4 B of cell
// id and 1 B of species, and writes back 28 B; per occupied cell it reads
// the 64-byte cell record (FP32 barycentric rows, neighbours), 16 B of dofs
// and four potentials, once per particle.
#include <cuda_runtime.h>

#include "pg_device.cuh"
#include "pg_walk.cuh"

namespace pg {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double block_sum_d(double v) {
    __shared__ double warp_part[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) warp_part[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (wid == 0) {
        s = lane < (int)(blockDim.x >> 5) ? warp_part[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    }
    __syncthreads();
    return s;
}

// Fixed-point deposit of one particle in cell c with barycentric
// coordinates l[] and the cell's dofs d (deposit_fixed's arithmetic).  agg:
// the lanes of the warp in the same cell add their contributions first
// (integer sums: the same bits as separate atomics) and the group's first
// lane issues the four atomics.
__device__ __forceinline__ void deposit_lambdas(bool agg, int c, const float l[4], int4 d, float q_scaled,
                                                unsigned long long *rho_fixed) {
    long long v0 = float_to_ll_rn(__fmul_rn(l[0], q_scaled)), v1 = float_to_ll_rn(__fmul_rn(l[1], q_scaled));
    long long v2 = float_to_ll_rn(__fmul_rn(l[2], q_scaled)), v3 = float_to_ll_rn(__fmul_rn(l[3], q_scaled));
    if (agg) {
        const unsigned peers = __match_any_sync(__activemask(), c);
        const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
        for (unsigned rest = peers & ~(1u << leader); rest; rest &= rest - 1) {
            const int src = __ffs(rest) - 1;
            const long long w0 = __shfl_sync(peers, v0, src), w1 = __shfl_sync(peers, v1, src);
            const long long w2 = __shfl_sync(peers, v2, src), w3 = __shfl_sync(peers, v3, src);
            if (lane == leader) { v0 += w0; v1 += w1; v2 += w2; v3 += w3; }
        }
        if (lane != leader) return;
    }
    atomicAdd(rho_fixed + d.x, (unsigned long long)v0);
    atomicAdd(rho_fixed + d.y, (unsigned long long)v1);
    atomicAdd(rho_fixed + d.z, (unsigned long long)v2);
    atomicAdd(rho_fixed + d.w, (unsigned long long)v3);
}

// Cell record of c: barycentric rows 0-2 and the neighbours (int bits).
struct CellRec {
    float4 r0, r1, r2, nb;
};
__device__ __forceinline__ CellRec load_rec(const DevMesh &m, int c) {
    const float4 *R = m.cell_f + 4 * (size_t)c;
    return CellRec{__ldg(R), __ldg(R + 1), __ldg(R + 2), __ldg(R + 3)};
}

template <bool PUSH, bool HAS_B, bool ACCEL, bool MOVE, bool PERIODIC, bool WALK, bool DEPOSIT>
__global__ void __launch_bounds__(512, 2) k_mixed(DevMesh m, DevParticles p, int64_t n_slots, MixedParams mp,
                                                   int max_steps, unsigned long long *__restrict__ rho_fixed,
                                                   DevState *__restrict__ st, double *__restrict__ partials) {
    float ke = 0.0f;   // this thread's particles in FP32 (~13 per thread), the block sum in FP64
    int retests = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n_use = slots_in_use(p, n_slots);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_use; i += stride) {
        int c = p.cell[i];
        if (c < 0) continue;
        const int s = p.sp[i];
        float x = p.xf[i], y = p.yf[i], z = p.zf[i];
        // the record and dofs of the particle's cell, loaded once for the
        // field, the walk's first cell and the deposit
        CellRec R;
        bool have_rec = false;
        int4 dd = make_int4(0, 0, 0, 0);
        bool have_d = false;
        if (PUSH || MOVE) {
            float vx = p.vxf[i], vy = p.vyf[i], vz = p.vzf[i];
            if (PUSH) {
                float4 E;
                if (mp.cg1) {
                    // CG1 vertex field interpolated at the FP32 position
                    R = load_rec(m, c);
                    have_rec = true;
                    const float l0 = fmaf(R.r0.w, z, fmaf(R.r0.z, y, fmaf(R.r0.y, x, R.r0.x)));
                    const float l1 = fmaf(R.r1.w, z, fmaf(R.r1.z, y, fmaf(R.r1.y, x, R.r1.x)));
                    const float l2 = fmaf(R.r2.w, z, fmaf(R.r2.z, y, fmaf(R.r2.y, x, R.r2.x)));
                    const float l3 = 1.0f - l0 - l1 - l2;
                    dd = __ldg(m.dofs + c);
                    have_d = true;
                    const float4 *V = reinterpret_cast<const float4 *>(m.Evf);
                    const float4 v0 = __ldg(V + dd.x), v1 = __ldg(V + dd.y), v2 = __ldg(V + dd.z), v3 = __ldg(V + dd.w);
                    E.x = fmaf(l3, v3.x, fmaf(l2, v2.x, fmaf(l1, v1.x, l0 * v0.x)));
                    E.y = fmaf(l3, v3.y, fmaf(l2, v2.y, fmaf(l1, v1.y, l0 * v0.y)));
                    E.z = fmaf(l3, v3.z, fmaf(l2, v2.z, fmaf(l1, v1.z, l0 * v0.z)));
                    E.w = 0.0f;
                } else if (mp.phi) {
                    R = load_rec(m, c);
                    have_rec = true;
                    dd = __ldg(m.dofs + c);
                    have_d = true;
                    E = dg0_field_f32(R.r0, R.r1, R.r2, dd, mp.phi, mp.E0[0], mp.E0[1], mp.E0[2]);
                } else {
                    E = __ldg(reinterpret_cast<const float4 *>(m.E_f) + c);
                }
                const float coef = mp.coef[s], hm = mp.half_m[s];
                if (ACCEL) {
                    const float ax = E.x * coef, ay = E.y * coef, az = E.z * coef;
                    ke += hm * fmaf(vx, vx + ax, fmaf(vy, vy + ay, vz * (vz + az)));
                    vx += ax; vy += ay; vz += az;
                } else {
                    const float hx = coef * E.x, hy = coef * E.y, hz = coef * E.z;
                    const float mx = vx + hx, my = vy + hy, mz = vz + hz;
                    ke += hm * fmaf(mx, mx, fmaf(my, my, mz * mz));
                    float px = mx, py = my, pz = mz;
                    if (HAS_B) {
                        const float t0 = mp.t[s][0], t1 = mp.t[s][1], t2 = mp.t[s][2];
                        const float s0 = mp.s[s][0], s1 = mp.s[s][1], s2 = mp.s[s][2];
                        const float rx = mx + (my * t2 - mz * t1);
                        const float ry = my + (mz * t0 - mx * t2);
                        const float rz = mz + (mx * t1 - my * t0);
                        px = mx + (ry * s2 - rz * s1);
                        py = my + (rz * s0 - rx * s2);
                        pz = mz + (rx * s1 - ry * s0);
                    }
                    vx = px + hx; vy = py + hy; vz = pz + hz;
                }
                p.vxf[i] = vx; p.vyf[i] = vy; p.vzf[i] = vz;
            }
            if (MOVE) {
                x = fmaf(mp.dt, vx, x); y = fmaf(mp.dt, vy, y); z = fmaf(mp.dt, vz, z);
                if (PERIODIC) {
                    x -= mp.Ld[0] * floorf(x / mp.Ld[0]);
                    y -= mp.Ld[1] * floorf(y / mp.Ld[1]);
                    z -= mp.Ld[2] * floorf(z / mp.Ld[2]);
                }
                p.xf[i] = x; p.yf[i] = y; p.zf[i] = z;
            }
        }
        float l[4];
        if (WALK) {
            // walk_mixed with the first cell's record already loaded; the
            // last cell's lambdas are the deposit's
            float e[4];
            int cc = c, end = kWalkFail;
            for (int it = 0; it < max_steps; ++it) {
                if (!have_rec) R = load_rec(m, cc);
                have_rec = false;
                lambdas_f32(R.r0, R.r1, R.r2, x, y, z, l, e);
                int next;
                if (facet_positive(m, cc, 0, l[0], e[0], x, y, z, retests)) next = __float_as_int(R.nb.x);
                else if (facet_positive(m, cc, 1, l[1], e[1], x, y, z, retests)) next = __float_as_int(R.nb.y);
                else if (facet_positive(m, cc, 2, l[2], e[2], x, y, z, retests)) next = __float_as_int(R.nb.z);
                else if (facet_positive(m, cc, 3, l[3], e[3], x, y, z, retests)) next = __float_as_int(R.nb.w);
                else { end = cc; break; }
                if (next < 0) { end = next; break; }
                cc = next;
            }
            if (end == kWalkFail) {
                raise_device_error(st, PG_ERR_WALK_LIMIT, i);
                continue;
            }
            if (end < 0) {
                const int tag = -end;
                atomicAdd(reinterpret_cast<unsigned long long *>(&st->absorbed[tag < kMaxTags ? tag : 0][s]), 1ull);
                atomicAdd(reinterpret_cast<unsigned long long *>(&st->live[s]), ~0ull);
                p.cell[i] = kDead;
                continue;
            }
            if (end != c) { p.cell[i] = end; c = end; have_d = false; }
        }
        if (DEPOSIT) {
            if (!WALK) {
                if (!have_rec) R = load_rec(m, c);
                l[0] = fmaf(R.r0.w, z, fmaf(R.r0.z, y, fmaf(R.r0.y, x, R.r0.x)));
                l[1] = fmaf(R.r1.w, z, fmaf(R.r1.z, y, fmaf(R.r1.y, x, R.r1.x)));
                l[2] = fmaf(R.r2.w, z, fmaf(R.r2.z, y, fmaf(R.r2.y, x, R.r2.x)));
                l[3] = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, l[0]), l[1]), l[2]);
            }
            if (!have_d) dd = __ldg(m.dofs + c);
            deposit_lambdas(mp.dep_agg != 0, c, l, dd, mp.q_scaled[s], rho_fixed);
        }
    }
    if (PUSH) {
        const double t = block_sum_d((double)ke);
        if (threadIdx.x == 0) partials[blockIdx.x] = t;
    }
    if (WALK && retests) atomicAdd(reinterpret_cast<unsigned long long *>(&st->retests), (unsigned long long)retests);
}

__global__ void k_sum_partials_m(const double *__restrict__ part, int n, double *__restrict__ out) {
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[i];
    const double s = block_sum_d(v);
    if (threadIdx.x == 0) *out = s;
}

__global__ void __launch_bounds__(kThreads) k_kinetic_mixed(DevParticles p, int64_t n_slots, MixedParams mp,
                                                           double *__restrict__ partials) {
    double ke = 0.0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n_use = slots_in_use(p, n_slots);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_use; i += stride) {
        if (p.cell[i] < 0) continue;
        const float hm = mp.half_m[p.sp[i]];
        const float vx = p.vxf[i], vy = p.vyf[i], vz = p.vzf[i];
        ke += (double)(hm * fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
    }
    const double s = block_sum_d(ke);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// rho = (sum in units of 2^-kFixedBits q_max) * q_max 2^-kFixedBits * dv_inv
__global__ void k_fixed_to_rho(const unsigned long long *__restrict__ fixed, const double *__restrict__ dv_inv,
                               double unit, int32_t n, double *__restrict__ rho_acc, double *__restrict__ rho) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = (double)(long long)fixed[i] * unit;
    if (rho_acc) rho_acc[i] = a;
    rho[i] = a * dv_inv[i];
}

// The mixed form's cell records: FP32 barycentric rows 0-2 and the
// neighbour ids (int bits in the fourth float4).
__global__ void k_float_tables(const double *__restrict__ bary, const int4 *__restrict__ nbr, int32_t nc,
                               float4 *__restrict__ cell_f) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const double *A = bary + 12 * (size_t)c;
    for (int k = 0; k < 3; ++k)
        cell_f[4 * (size_t)c + k] = make_float4((float)A[4 * k], (float)A[4 * k + 1], (float)A[4 * k + 2], (float)A[4 * k + 3]);
    const int4 nb = nbr[c];
    cell_f[4 * (size_t)c + 3] = make_float4(__int_as_float(nb.x), __int_as_float(nb.y), __int_as_float(nb.z),
                                            __int_as_float(nb.w));
}

inline int grid_for(int64_t n, int max_blocks) {
    int64_t g = (n + kThreads - 1) / kThreads;
    if (g < 1) g = 1;
    if (g > max_blocks) g = max_blocks;
    return (int)g;
}

}  // namespace

void launch_mixed_pass(const DevMesh &m, const DevParticles &p, int64_t n_slots, const MixedParams &mp, bool push,
                       bool move, bool walk, bool deposit, int max_steps, unsigned long long *rho_fixed,
                       DevState *state, double *partials, int nblocks, double *ke_out, cudaStream_t st) {
    if (n_slots <= 0) return;
    const int threads = mp.threads > 0 ? mp.threads : kThreads;
    int64_t gg = (n_slots + threads - 1) / threads;
    const int64_t cap = push ? nblocks : (1 << 20);
    const int g = (int)(gg < 1 ? 1 : (gg > cap ? cap : gg));
    count_launches(push ? 2 : 1);
#define PG_MIX(PU, HB, AC, MO, PE, WA, DE) \
    k_mixed<PU, HB, AC, MO, PE, WA, DE><<<g, threads, 0, st>>>(m, p, n_slots, mp, max_steps, rho_fixed, state, partials)
    if (push && move && walk && deposit) {
        if (mp.accel) { if (mp.periodic) PG_MIX(true, false, true, true, true, true, true); else PG_MIX(true, false, true, true, false, true, true); }
        else if (mp.has_B) { if (mp.periodic) PG_MIX(true, true, false, true, true, true, true); else PG_MIX(true, true, false, true, false, true, true); }
        else { if (mp.periodic) PG_MIX(true, false, false, true, true, true, true); else PG_MIX(true, false, false, true, false, true, true); }
    } else if (push) {
        if (mp.accel) PG_MIX(true, false, true, false, false, false, false);
        else if (mp.has_B) PG_MIX(true, true, false, false, false, false, false);
        else PG_MIX(true, false, false, false, false, false, false);
    } else if (move) {
        if (mp.periodic) PG_MIX(false, false, false, true, true, false, false);
        else PG_MIX(false, false, false, true, false, false, false);
    } else if (walk) {
        PG_MIX(false, false, false, false, false, true, false);
    } else if (deposit) {
        PG_MIX(false, false, false, false, false, false, true);
    }
#undef PG_MIX
    if (push) k_sum_partials_m<<<1, 1024, 0, st>>>(partials, g, ke_out);
}

void launch_kinetic_mixed(const DevParticles &p, int64_t n_slots, const MixedParams &mp, double *partials, int nblocks,
                          double *ke_out, cudaStream_t st) {
    const int g = grid_for(n_slots, nblocks);
    count_launches(2);
    k_kinetic_mixed<<<g, kThreads, 0, st>>>(p, n_slots, mp, partials);
    k_sum_partials_m<<<1, 1024, 0, st>>>(partials, g, ke_out);
}

void launch_fixed_to_rho(const unsigned long long *fixed, const double *dv_inv, double unit, int32_t n,
                         double *rho_acc, double *rho, cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1);
    k_fixed_to_rho<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(fixed, dv_inv, unit, n, rho_acc, rho);
}

void launch_float_tables(const double *bary, const int4 *nbr, int32_t nc, float4 *cell_f, cudaStream_t st) {
    count_launches(1);
    k_float_tables<<<(nc + kThreads - 1) / kThreads, kThreads, 0, st>>>(bary, nbr, nc, cell_f);
}

}  // namespace pg
