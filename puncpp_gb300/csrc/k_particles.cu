// FP64 particle kernels: DG0 or CG1 field gather + Boris/accel push, move, facet-walk
// relocation with absorption, CG1 deposition, point location, cell sort.
//
// Built with --fmad=false: every multiply and add rounds on its own, in the
// operation order of the reference (cited per function), so positions,
// velocities and cell indices equal those of a CPU evaluation bit for bit.
#include <cuda_runtime.h>

#include <atomic>

#include "pg_device.cuh"
#include "pg_walk.cuh"

namespace pg {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double warp_part[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) warp_part[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        s = lane < nw ? warp_part[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    }
    __syncthreads();
    return s;  // valid in thread 0
}

// All four plane values <= 0: the point is in the cell (the walk would stay).
__device__ __forceinline__ bool inside_fp64(const DevMesh &m, double x, double y, double z, int c) {
    const double2 *P = reinterpret_cast<const double2 *>(m.planes) + 8 * (size_t)c;
    for (int f = 0; f < 4; ++f) {
        const double2 a = __ldg(P + 2 * f), b = __ldg(P + 2 * f + 1);
        double d = a.x + a.y * x; d = d + b.x * y; d = d + b.y * z;
        if (d > 0) return false;
    }
    return true;
}

// One pass over the particle slots doing any of push, move, walk and deposit.
template <bool PUSH, bool HAS_B, bool ACCEL, bool MOVE, bool PERIODIC, bool WALK, bool DEPOSIT>
__global__ void __launch_bounds__(512) k_particles(DevMesh m, DevParticles p, int64_t n_slots, PushParams pp,
                                                       MoveParams mp, int max_steps, const double *__restrict__ qsp,
                                                       double *__restrict__ rho_acc, DevState *__restrict__ st,
                                                       double *__restrict__ partials) {
    double ke = 0.0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n_use = slots_in_use(p, n_slots);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_use; i += stride) {
        int c = p.cell[i];
        if (c < 0) continue;
        const int s = p.sp[i];
        double x = p.x[i], y = p.y[i], z = p.z[i];
        if (PUSH || MOVE) {
            double vx = p.vx[i], vy = p.vy[i], vz = p.vz[i];
            if (PUSH) {
                double ex, ey, ez;
                if (pp.cg1) {
                    // accel_cg1 / boris_cg1 (punc/include/punc/pusher.h:154-201, 282-372):
                    // Ei = sum_i coeffs[i] * values[j*4 + i] over the cell's vertices
                    double l0, l1, l2, l3;
                    barycentric_fp64(m, c, x, y, z, l0, l1, l2, l3);
                    const int4 d = __ldg(m.dofs + c);
                    const double2 *V = reinterpret_cast<const double2 *>(m.Ev);
                    const double2 a0 = __ldg(V + 2 * (size_t)d.x), b0 = __ldg(V + 2 * (size_t)d.x + 1);
                    const double2 a1 = __ldg(V + 2 * (size_t)d.y), b1 = __ldg(V + 2 * (size_t)d.y + 1);
                    const double2 a2 = __ldg(V + 2 * (size_t)d.z), b2 = __ldg(V + 2 * (size_t)d.z + 1);
                    const double2 a3 = __ldg(V + 2 * (size_t)d.w), b3 = __ldg(V + 2 * (size_t)d.w + 1);
                    ex = l0 * a0.x; ex = ex + l1 * a1.x; ex = ex + l2 * a2.x; ex = ex + l3 * a3.x;
                    ey = l0 * a0.y; ey = ey + l1 * a1.y; ey = ey + l2 * a2.y; ey = ey + l3 * a3.y;
                    ez = l0 * b0.x; ez = ez + l1 * b1.x; ez = ez + l2 * b2.x; ez = ez + l3 * b3.x;
                } else {
                    const double2 *Ec = reinterpret_cast<const double2 *>(m.E) + 2 * (size_t)c;
                    const double2 e01 = __ldg(Ec);
                    const double2 e2_ = __ldg(Ec + 1);
                    ex = e01.x; ey = e01.y; ez = e2_.x;
                }
                const double coef = pp.coef[s], hm = pp.half_m[s];
                if (ACCEL) {
                    // accel (punc/include/punc/pusher.h:66-130): Ei *= dt*(q/m);
                    // KE += 0.5*m*v*(v+Ei); v += Ei.
                    const double ax = ex * coef, ay = ey * coef, az = ez * coef;
                    ke += hm * vx * (vx + ax);
                    ke += hm * vy * (vy + ay);
                    ke += hm * vz * (vz + az);
                    vx = vx + ax; vy = vy + ay; vz = vz + az;
                } else {
                    // boris (punc/include/punc/pusher.h:397-510).
                    const double hx = coef * ex, hy = coef * ey, hz = coef * ez;
                    const double mx = vx + hx, my = vy + hy, mz = vz + hz;
                    ke += hm * mx * mx;
                    ke += hm * my * my;
                    ke += hm * mz * mz;
                    double px = mx, py = my, pz = mz;
                    if (HAS_B) {
                        const double t0 = pp.t[s][0], t1 = pp.t[s][1], t2 = pp.t[s][2];
                        const double s0 = pp.s[s][0], s1 = pp.s[s][1], s2 = pp.s[s][2];
                        const double cx = my * t2 - mz * t1;
                        const double cy = -mx * t2 + mz * t0;
                        const double cz = mx * t1 - my * t0;
                        const double rx = mx + cx, ry = my + cy, rz = mz + cz;
                        const double dx = ry * s2 - rz * s1;
                        const double dy = -rx * s2 + rz * s0;
                        const double dz = rx * s1 - ry * s0;
                        px = mx + dx; py = my + dy; pz = mz + dz;
                    }
                    vx = px + hx; vy = py + hy; vz = pz + hz;
                }
                p.vx[i] = vx; p.vy[i] = vy; p.vz[i] = vz;
            }
            if (MOVE) {
                // move / move_periodic (punc/include/punc/pusher.h:648-681).
                x = x + mp.dt * vx; y = y + mp.dt * vy; z = z + mp.dt * vz;
                if (PERIODIC) {
                    x = x - mp.Ld[0] * floor(x / mp.Ld[0]);
                    y = y - mp.Ld[1] * floor(y / mp.Ld[1]);
                    z = z - mp.Ld[2] * floor(z / mp.Ld[2]);
                }
                p.x[i] = x; p.y[i] = y; p.z[i] = z;
            }
        }
        if (WALK) {
            // Population::update (punc/include/punc/population.h:641-699).
            const int nc = walk_fp64(m, x, y, z, c, max_steps);
            if (nc == kWalkFail) {
                raise_device_error(st, PG_ERR_WALK_LIMIT, i);
                continue;
            }
            if (nc < 0) {
                const int tag = -nc;
                atomicAdd(reinterpret_cast<unsigned long long *>(&st->absorbed[tag < kMaxTags ? tag : 0][s]), 1ull);
                atomicAdd(reinterpret_cast<unsigned long long *>(&st->live[s]), ~0ull);
                p.cell[i] = kDead;
                continue;
            }
            if (nc != c) { p.cell[i] = nc; c = nc; }
        }
        if (DEPOSIT) {
            // distribute_cg1 (punc/include/punc/distributor.h:168-210): q * lambda_i.
            double l0, l1, l2, l3;
            barycentric_fp64(m, c, x, y, z, l0, l1, l2, l3);
            const double q = qsp[s];
            const int4 d = __ldg(m.dofs + c);
            atomicAdd(rho_acc + d.x, q * l0);
            atomicAdd(rho_acc + d.y, q * l1);
            atomicAdd(rho_acc + d.z, q * l2);
            atomicAdd(rho_acc + d.w, q * l3);
        }
    }
    if (PUSH) {
        const double s = block_sum(ke);
        if (threadIdx.x == 0) partials[blockIdx.x] = s;
    }
}

__global__ void k_sum_partials(const double *__restrict__ part, int n, double *__restrict__ out) {
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[i];
    const double s = block_sum(v);
    if (threadIdx.x == 0) *out = s;
}

// kinetic_energy (punc/include/punc/diagnostics.h:248-265).
__global__ void __launch_bounds__(kThreads) k_kinetic(DevParticles p, int64_t n_slots, PushParams pp,
                                                     double *__restrict__ partials) {
    double ke = 0.0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n_use = slots_in_use(p, n_slots);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_use; i += stride) {
        if (p.cell[i] < 0) continue;
        const double hm = pp.half_m[p.sp[i]];
        const double vx = p.vx[i], vy = p.vy[i], vz = p.vz[i];
        ke += hm * vx * vx;
        ke += hm * vy * vy;
        ke += hm * vz * vz;
    }
    const double s = block_sum(ke);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// Point location over the bin grid: first cell of the point's bin (in
// ascending cell order) whose four plane values are all <= 0.
__global__ void k_locate(DevMesh m, const double *__restrict__ xyz, int64_t n, int32_t *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    const double u[3] = {x, y, z};
    int b[3];
    for (int j = 0; j < 3; ++j) {
        const double f = floor((u[j] - m.lo[j]) / m.bin_h[j]);
        if (!(f >= -1.0 && f <= (double)m.nbin[j])) { out[i] = -1; return; }
        b[j] = f < 0 ? 0 : (f >= m.nbin[j] ? m.nbin[j] - 1 : (int)f);
    }
    const int64_t bin = ((int64_t)b[0] * m.nbin[1] + b[1]) * m.nbin[2] + b[2];
    int found = -1;
    for (int64_t k = m.bin_ptr[bin]; k < m.bin_ptr[bin + 1]; ++k) {
        const int c = m.bin_cells[k];
        if (c < m.loc_lo || c >= m.loc_hi) continue;
        if (inside_fp64(m, x, y, z, c)) { found = c; break; }
    }
    out[i] = found;
}

// Single-point walks of Population (punc/include/punc/population.h:454-570)
// from given cells: mode 0 relocate_fast (the first facet with a positive
// plane value), mode 1 relocate and relocate_stat (the facet of the largest
// plane value, the first of equal ones; the walk stays only when every value
// is negative).  Plane values summed left to right as the reference.
// out: the final cell or -tag; cross: facets crossed; a walk that reaches
// max_steps reports kWalkFail.
__global__ void k_relocate(DevMesh m, const double *__restrict__ xyz, const int32_t *__restrict__ start, int64_t n,
                           int mode, int max_steps, int32_t *__restrict__ out, int32_t *__restrict__ cross) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    int c = start[i], k = 0, end = kWalkFail;
    for (int it = 0; it < max_steps; ++it) {
        const double *P = m.planes + 16 * (size_t)c;
        const int4 nb = __ldg(m.nbr + c);
        const int nbv[4] = {nb.x, nb.y, nb.z, nb.w};
        double d[4];
#pragma unroll
        for (int f = 0; f < 4; ++f) d[f] = plane64(P[4 * f], P[4 * f + 1], P[4 * f + 2], P[4 * f + 3], x, y, z);
        int f = -1;
        if (mode == 0) {
            for (int q = 0; q < 4; ++q)
                if (d[q] > 0) { f = q; break; }
        } else {
            int a = 0;
            for (int q = 1; q < 4; ++q)
                if (d[q] > d[a]) a = q;
            f = d[a] < 0 ? -1 : a;
        }
        if (f < 0) { end = c; break; }
        ++k;
        if (nbv[f] < 0) { end = nbv[f]; break; }
        c = nbv[f];
    }
    out[i] = end;
    if (cross) cross[i] = k;
}

// x <- 2 x - x_prev, x_prev <- old x (linear extrapolation of the last two solutions).
__global__ void k_extrapolate(double *__restrict__ x, double *__restrict__ x_prev, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xn = x[i];
    x[i] = 2.0 * xn - x_prev[i];
    x_prev[i] = xn;
}

__global__ void k_scale(const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ o, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) o[i] = a[i] * b[i];
}

// ---- exclusive scan of int64 (reduce, scan the block sums, rescan) --------
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int64_t kScanTile = (int64_t)kScanThreads * kScanItems;

__device__ int64_t block_exclusive_scan(int64_t v, int64_t &total) {
    __shared__ int64_t wsum[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        int64_t w = lane < nw ? wsum[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < nw) wsum[lane] = w;
    }
    __syncthreads();
    const int64_t before = wid > 0 ? wsum[wid - 1] : 0;
    total = wsum[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before + incl - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int64_t *__restrict__ in, int64_t n,
                                                              int64_t *__restrict__ sums) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t v = 0;
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + (int64_t)threadIdx.x * kScanItems + k;
        if (i < n) v += in[i];
    }
    int64_t total;
    block_exclusive_scan(v, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int64_t *__restrict__ sums, int64_t nb) {
    int64_t carry = 0;
    for (int64_t base = 0; base < nb; base += kScanThreads) {
        const int64_t i = base + threadIdx.x;
        const int64_t v = i < nb ? sums[i] : 0;
        int64_t total;
        const int64_t ex = block_exclusive_scan(v, total);
        if (i < nb) sums[i] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int64_t *__restrict__ in, int64_t n,
                                                             const int64_t *__restrict__ sums,
                                                             int64_t *__restrict__ out) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t loc[kScanItems];
    int64_t v = 0;
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + (int64_t)threadIdx.x * kScanItems + k;
        loc[k] = i < n ? in[i] : 0;
        v += loc[k];
    }
    int64_t total;
    int64_t run = block_exclusive_scan(v, total) + sums[blockIdx.x];
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + (int64_t)threadIdx.x * kScanItems + k;
        if (i < n) out[i] = run;
        run += loc[k];
    }
}

__global__ void k_sort_hist(DevParticles p, int64_t n_slots, int64_t *__restrict__ hist) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n_use = slots_in_use(p, n_slots);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_use; i += stride) {
        const int c = p.cell[i];
        if (c >= 0) atomicAdd(reinterpret_cast<unsigned long long *>(hist + c), 1ull);
    }
}

template <bool MIXED>
__global__ void k_sort_scatter(DevParticles s, DevParticles d, int64_t n_slots, int64_t *__restrict__ cursor) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n_use = slots_in_use(s, n_slots);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_use; i += stride) {
        const int c = s.cell[i];
        if (c < 0) continue;
        const int64_t j = (int64_t)atomicAdd(reinterpret_cast<unsigned long long *>(cursor + c), 1ull);
        if (MIXED) {
            d.xf[j] = s.xf[i]; d.yf[j] = s.yf[i]; d.zf[j] = s.zf[i];
            d.vxf[j] = s.vxf[i]; d.vyf[j] = s.vyf[i]; d.vzf[j] = s.vzf[i];
        } else {
            d.x[j] = s.x[i]; d.y[j] = s.y[i]; d.z[j] = s.z[i];
            d.vx[j] = s.vx[i]; d.vy[j] = s.vy[i]; d.vz[j] = s.vz[i];
        }
        d.cell[j] = c; d.sp[j] = s.sp[i]; d.pid[j] = s.pid[i];
    }
}

inline int grid_for(int64_t n, int max_blocks) {
    int64_t g = (n + kThreads - 1) / kThreads;
    if (g < 1) g = 1;
    if (g > max_blocks) g = max_blocks;
    return (int)g;
}

}  // namespace

static std::atomic<long long> g_launches{0};
void count_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches_so_far() { return g_launches.load(); }

int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

void launch_push(const DevMesh &m, const DevParticles &p, int64_t n_slots, const PushParams &pp,
                 double *partials, int nblocks, double *ke_out, cudaStream_t st) {
    const int g = grid_for(n_slots, nblocks);
    MoveParams mp{};
    count_launches(2);
    if (pp.accel)
        k_particles<true, false, true, false, false, false, false><<<g, kThreads, 0, st>>>(m, p, n_slots, pp, mp, 0, nullptr, nullptr, nullptr, partials);
    else if (pp.has_B)
        k_particles<true, true, false, false, false, false, false><<<g, kThreads, 0, st>>>(m, p, n_slots, pp, mp, 0, nullptr, nullptr, nullptr, partials);
    else
        k_particles<true, false, false, false, false, false, false><<<g, kThreads, 0, st>>>(m, p, n_slots, pp, mp, 0, nullptr, nullptr, nullptr, partials);
    k_sum_partials<<<1, 1024, 0, st>>>(partials, g, ke_out);
}

void launch_move(const DevParticles &p, int64_t n_slots, const MoveParams &mp, cudaStream_t st) {
    const int g = grid_for(n_slots, 1 << 20);
    DevMesh m{};
    PushParams pp{};
    count_launches(1);
    if (mp.periodic)
        k_particles<false, false, false, true, true, false, false><<<g, kThreads, 0, st>>>(m, p, n_slots, pp, mp, 0, nullptr, nullptr, nullptr, nullptr);
    else
        k_particles<false, false, false, true, false, false, false><<<g, kThreads, 0, st>>>(m, p, n_slots, pp, mp, 0, nullptr, nullptr, nullptr, nullptr);
}

void launch_update(const DevMesh &m, const DevParticles &p, int64_t n_slots, int max_steps, DevState *state,
                   cudaStream_t st) {
    const int g = grid_for(n_slots, 1 << 20);
    PushParams pp{};
    MoveParams mp{};
    count_launches(1);
    k_particles<false, false, false, false, false, true, false><<<g, kThreads, 0, st>>>(m, p, n_slots, pp, mp, max_steps, nullptr, nullptr, state, nullptr);
}

void launch_deposit(const DevMesh &m, const DevParticles &p, int64_t n_slots, const double *q_species,
                    double *rho_acc, cudaStream_t st) {
    const int g = grid_for(n_slots, 1 << 20);
    PushParams pp{};
    MoveParams mp{};
    count_launches(1);
    k_particles<false, false, false, false, false, false, true><<<g, kThreads, 0, st>>>(m, p, n_slots, pp, mp, 0, q_species, rho_acc, nullptr, nullptr);
}

void launch_fused_step(const DevMesh &m, const DevParticles &p, int64_t n_slots, const PushParams &pp,
                       const MoveParams &mp, int max_steps, const double *q_species, double *rho_acc,
                       DevState *state, double *partials, int nblocks, double *ke_out, cudaStream_t st) {
    const int threads = pp.threads > 0 ? pp.threads : kThreads;
    int64_t gg = (n_slots + threads - 1) / threads;
    const int g = (int)(gg < 1 ? 1 : (gg > nblocks ? nblocks : gg));
    count_launches(2);
#define PG_FUSED(HB, AC, PER)                                                                            \
    k_particles<true, HB, AC, true, PER, true, true><<<g, threads, 0, st>>>(m, p, n_slots, pp, mp, max_steps, \
                                                                           q_species, rho_acc, state, partials)
    if (pp.accel) {
        if (mp.periodic) PG_FUSED(false, true, true); else PG_FUSED(false, true, false);
    } else if (pp.has_B) {
        if (mp.periodic) PG_FUSED(true, false, true); else PG_FUSED(true, false, false);
    } else {
        if (mp.periodic) PG_FUSED(false, false, true); else PG_FUSED(false, false, false);
    }
#undef PG_FUSED
    k_sum_partials<<<1, 1024, 0, st>>>(partials, g, ke_out);
}

void launch_kinetic(const DevParticles &p, int64_t n_slots, const double *half_m, double *partials, int nblocks,
                    double *ke_out, cudaStream_t st) {
    PushParams pp{};
    for (int s = 0; s < kMaxSpecies; ++s) pp.half_m[s] = half_m[s];
    const int g = grid_for(n_slots, nblocks);
    count_launches(2);
    k_kinetic<<<g, kThreads, 0, st>>>(p, n_slots, pp, partials);
    k_sum_partials<<<1, 1024, 0, st>>>(partials, g, ke_out);
}

void launch_locate(const DevMesh &m, const double *xyz, int64_t n, int32_t *cells, cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1);
    k_locate<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, st>>>(m, xyz, n, cells);
}

void launch_relocate(const DevMesh &m, const double *xyz, const int32_t *start, int64_t n, int mode, int max_steps,
                     int32_t *out, int32_t *cross, cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1);
    k_relocate<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, st>>>(m, xyz, start, n, mode, max_steps, out,
                                                                            cross);
}

void launch_scale(const double *a, const double *b, double *out, int64_t n, cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1);
    k_scale<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, st>>>(a, b, out, n);
}

void launch_extrapolate(double *x, double *x_prev, int64_t n, cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1);
    k_extrapolate<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, st>>>(x, x_prev, n);
}

int64_t scan_tmp_size(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

void launch_scan_i64(const int64_t *in, int64_t *out, int64_t n, int64_t *tmp, cudaStream_t st) {
    if (n <= 0) return;
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    count_launches(3);
    k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, tmp);
    k_scan_sums<<<1, kScanThreads, 0, st>>>(tmp, nb);
    k_scan_apply<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, tmp, out);
}

void launch_sort_hist(const DevParticles &p, int64_t n_slots, int64_t *hist, cudaStream_t st) {
    if (n_slots <= 0) return;
    count_launches(1);
    k_sort_hist<<<grid_for(n_slots, sm_count() * 16), kThreads, 0, st>>>(p, n_slots, hist);
}

void launch_sort_scatter(const DevParticles &src, const DevParticles &dst, int64_t n_slots, int64_t *cursor,
                         cudaStream_t st) {
    if (n_slots <= 0) return;
    count_launches(1);
    if (src.xf)
        k_sort_scatter<true><<<grid_for(n_slots, sm_count() * 16), kThreads, 0, st>>>(src, dst, n_slots, cursor);
    else
        k_sort_scatter<false><<<grid_for(n_slots, sm_count() * 16), kThreads, 0, st>>>(src, dst, n_slots, cursor);
}

}  // namespace pg
