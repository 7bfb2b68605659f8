// PCG preconditioned by one smoothed-aggregation AMG V-cycle per iteration,
// all in one cooperative launch.
//
// Krylov recurrence in FP32 with the solution, inner products and
// true-residual replacements in FP64 (as k_pcg_rel), stopping on the FP64
// true residual ||b - A x|| <= max(rtol ||b||, atol).
//
// The V-cycle (one weighted-Jacobi sweep from zero before the coarse
// correction and one after, Galerkin coarse operators, dense coarsest
// inverse) is applied in the algebraically identical form
//     B_l b = W_l b + S_l B_{l+1} S_l^T b,   W = w D^-1 (2 I - A w D^-1),
//     S = (I - w D^-1 A) P,
// with the last restriction and the coarse solve in one product
// (G = C^-1 S^T) and the up-sweep of levels >= 1 collapsed into one product
// (U1 = [S_1 | S_1 S_2 | ...]): L + 1 grid-wide phases for L >= 2 levels
// above the coarsest.  The product A z of the search direction update is
// folded into the next matrix phase (A p = A z + beta A p_old) and r.z into
// the last V-cycle phase: an iteration is L + 3 grid barriers.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "pg_device.cuh"
#include "pg_reduce.cuh"

namespace cg = cooperative_groups;

namespace pg {

namespace {

// Vectors written inside the kernel are read with plain (L1-cached) loads
// only after a grid barrier, whose acquire makes the other blocks' writes
// visible; never through the read-only path (__ldg).
//
// epi(i, sum_j S_ij xv(j)) for every row i of S, spread over the whole grid.
// SELL operators take one thread per row, two rows at a time; CSR operators g
// lanes per row, reduced by warp shuffles (g <= 32) and through shared memory
// (g = 64..512, the warps of one block).  The loads of four entries are
// issued before their products so that a lane keeps several gathers in
// flight (the kernel runs at 32 warps per SM and is latency-bound otherwise).
// Every thread of the grid must call this (the CSR path runs the same number
// of rounds in all lanes so the shuffles are full-warp).
// This lane's share (entries lane, lane + g, ...) of row i of a CSR operator,
// four entries' loads issued before their products.
template <class XV>
__device__ __forceinline__ float csr_lane_sum(const SpOp &S, int i, int lane, int g, XV xv) {
    const int64_t k0 = __ldg(S.ptr + i);
    const int len = (int)(__ldg(S.ptr + i + 1) - k0);
    const int32_t *cp = S.col + k0;
    const float *vp = S.val + k0;
    float s0 = 0.0f, s1 = 0.0f;
    int k = lane;
    for (; k + 3 * g < len; k += 4 * g) {
        const int c0 = __ldg(cp + k), c1 = __ldg(cp + k + g);
        const int c2 = __ldg(cp + k + 2 * g), c3 = __ldg(cp + k + 3 * g);
        const float v0 = __ldg(vp + k), v1 = __ldg(vp + k + g);
        const float v2 = __ldg(vp + k + 2 * g), v3 = __ldg(vp + k + 3 * g);
        const float x0 = xv(c0), x1 = xv(c1), x2 = xv(c2), x3 = xv(c3);
        s0 = fmaf(v0, x0, s0);
        s1 = fmaf(v1, x1, s1);
        s0 = fmaf(v2, x2, s0);
        s1 = fmaf(v3, x3, s1);
    }
    for (; k < len; k += g) s0 = fmaf(__ldg(vp + k), xv(__ldg(cp + k)), s0);
    return s0 + s1;
}

// Two rows' lane shares at once (row ib may be absent: ib < 0), so that a
// lane keeps four gathers in flight across the two rows.
template <class XV>
__device__ __forceinline__ void csr_lane_sum2(const SpOp &S, int ia, int ib, int lane, int g, XV xv, float &ra,
                                              float &rb) {
    const int64_t ka = __ldg(S.ptr + ia);
    const int la = (int)(__ldg(S.ptr + ia + 1) - ka);
    int64_t kb = 0;
    int lb = 0;
    if (ib >= 0) {
        kb = __ldg(S.ptr + ib);
        lb = (int)(__ldg(S.ptr + ib + 1) - kb);
    }
    const int32_t *ca = S.col + ka, *cb = S.col + kb;
    const float *va = S.val + ka, *vb = S.val + kb;
    const int len = la > lb ? la : lb;
    float sa = 0.0f, sb = 0.0f;
    for (int k = lane; k < len; k += 2 * g) {
        const int k1 = k + g;
        const int c0 = k < la ? __ldg(ca + k) : -1, c1 = k1 < la ? __ldg(ca + k1) : -1;
        const int d0 = k < lb ? __ldg(cb + k) : -1, d1 = k1 < lb ? __ldg(cb + k1) : -1;
        const float v0 = k < la ? __ldg(va + k) : 0.0f, v1 = k1 < la ? __ldg(va + k1) : 0.0f;
        const float w0 = k < lb ? __ldg(vb + k) : 0.0f, w1 = k1 < lb ? __ldg(vb + k1) : 0.0f;
        const float x0 = c0 >= 0 ? xv(c0) : 0.0f, x1 = c1 >= 0 ? xv(c1) : 0.0f;
        const float y0 = d0 >= 0 ? xv(d0) : 0.0f, y1 = d1 >= 0 ? xv(d1) : 0.0f;
        sa = fmaf(v0, x0, sa);
        sb = fmaf(w0, y0, sb);
        sa = fmaf(v1, x1, sa);
        sb = fmaf(w1, y1, sb);
    }
    ra = sa;
    rb = sb;
}

template <class XV, class EPI>
__device__ __forceinline__ void apply(const SpOp &S, XV xv, EPI epi, int t0, int ts) {
    if (S.g == 1) {
        for (int i = t0; i < S.n; i += 2 * ts) {
            const int i2 = i + ts;
            const int64_t ba = __ldg(S.ptr + (i >> 5)) + (i & 31);
            const int wa = __ldg(S.swidth + (i >> 5));
            const bool two = i2 < S.n;
            const int64_t bb = two ? __ldg(S.ptr + (i2 >> 5)) + (i2 & 31) : 0;
            const int wb = two ? __ldg(S.swidth + (i2 >> 5)) : 0;
            float sa = 0.0f, sb = 0.0f;
            const int w = wa > wb ? wa : wb;
            for (int k = 0; k < w; k += 2) {
                // entries k, k+1 of both rows (padding entries are zero)
                const bool a0 = k < wa, a1 = k + 1 < wa, b0 = k < wb, b1 = k + 1 < wb;
                const int64_t oa = ba + 32 * k, ob = bb + 32 * k;
                const int ca0 = a0 ? __ldg(S.col + oa) : 0, ca1 = a1 ? __ldg(S.col + oa + 32) : 0;
                const int cb0 = b0 ? __ldg(S.col + ob) : 0, cb1 = b1 ? __ldg(S.col + ob + 32) : 0;
                const float va0 = a0 ? __ldg(S.val + oa) : 0.0f, va1 = a1 ? __ldg(S.val + oa + 32) : 0.0f;
                const float vb0 = b0 ? __ldg(S.val + ob) : 0.0f, vb1 = b1 ? __ldg(S.val + ob + 32) : 0.0f;
                const float xa0 = a0 ? xv(ca0) : 0.0f, xa1 = a1 ? xv(ca1) : 0.0f;
                const float xb0 = b0 ? xv(cb0) : 0.0f, xb1 = b1 ? xv(cb1) : 0.0f;
                sa = fmaf(va0, xa0, sa);
                sb = fmaf(vb0, xb0, sb);
                sa = fmaf(va1, xa1, sa);
                sb = fmaf(vb1, xb1, sb);
            }
            epi(i, sa);
            if (two) epi(i2, sb);
        }
    } else if (S.g <= 32) {
        const int g = S.g;
        const int lane = t0 & (g - 1);
        const int grp = t0 / g, ngrp = ts / g;
        const int rounds = (S.n + ngrp - 1) / ngrp;
        for (int t = 0; t < rounds; t += 2) {
            // rounds t and t + 1 together
            const int i = grp + t * ngrp, i2 = i + ngrp;
            float s = 0.0f, s2 = 0.0f;
            if (i < S.n) csr_lane_sum2(S, i, i2 < S.n ? i2 : -1, lane, g, xv, s, s2);
            for (int o = g >> 1; o > 0; o >>= 1) {
                s += __shfl_xor_sync(0xffffffffu, s, o);
                s2 += __shfl_xor_sync(0xffffffffu, s2, o);
            }
            if (lane == 0 && i < S.n) epi(i, s);
            if (lane == 0 && i2 < S.n) epi(i2, s2);
        }
    } else {
        // g / 32 warps of one block per row; partial sums meet in shared memory
        __shared__ float red[kPcgThreads / 32];
        const int g = S.g;
        const int per_block = blockDim.x / g;
        const int lane = threadIdx.x & (g - 1);
        const int grp = blockIdx.x * per_block + threadIdx.x / g;
        const int ngrp = gridDim.x * per_block;
        const int rounds = (S.n + ngrp - 1) / ngrp;
        for (int t = 0; t < rounds; ++t) {
            const int i = grp + t * ngrp;
            float s = i < S.n ? csr_lane_sum(S, i, lane, g, xv) : 0.0f;
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
            __syncthreads();
            if (lane == 0 && i < S.n) {
                float tot = 0.0f;
                for (int w = 0; w < g / 32; ++w) tot += red[(threadIdx.x >> 5) + w];
                epi(i, tot);
            }
            __syncthreads();
        }
    }
}

// z = B r over the whole grid, r complete on entry; returns this thread's
// share of r.z.  Level 0's b is r.
__device__ double vcycle(const AmgDev &M, const float *r, float *z, cg::grid_group &grid, int t0, int ts) {
    const int L = M.nlev - 1;
    double rz = 0.0;
    if (L == 0) {
        apply(M.cinv, [=](int j) { return r[j]; },
              [&](int i, float s) { z[i] = s; rz = fma((double)s, (double)r[i], rz); }, t0, ts);
        return rz;
    }
    for (int l = 0; l < L; ++l) {
        const float *b = l == 0 ? r : M.lev[l].b;
        const float om = M.lev[l].omega;
        const float *dinv = M.lev[l].dinv;
        float *t = M.lev[l].t;
        apply(M.lev[l].A, [=](int j) { return om * __ldg(dinv + j) * b[j]; },
              [=](int i, float s) { t[i] = om * __ldg(dinv + i) * (2.0f * b[i] - s); }, t0, ts);
        if (l < L - 1) {
            float *bn = M.lev[l + 1].b;
            apply(M.lev[l].ST, [=](int j) { return b[j]; }, [=](int i, float s) { bn[i] = s; }, t0, ts);
        } else {
            float *yL = M.yL;
            apply(M.G, [=](int j) { return b[j]; }, [=](int i, float s) { yL[i] = s; }, t0, ts);
        }
        grid.sync();
    }
    const float *yup = M.yL;
    if (L >= 2) {
        const float *t1 = M.lev[1].t, *st = M.stack;
        float *y1 = M.y1;
        apply(M.U1, [=](int j) { return st[j]; }, [=](int i, float s) { y1[i] = t1[i] + s; }, t0, ts);
        grid.sync();
        yup = M.y1;
    }
    const float *tz = M.lev[0].t;
    apply(M.S0, [=](int j) { return yup[j]; },
          [&](int i, float s) {
              const float zi = tz[i] + s;
              z[i] = zi;
              rz = fma((double)zi, (double)r[i], rz);
          }, t0, ts);
    return rz;
}

__global__ void __launch_bounds__(kPcgThreads, 2) k_pcg_amg(PcgArgs a, AmgDev M) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[2 * kPcgThreads + 16];
    __shared__ double scal[4];
    const int nb = gridDim.x;
    const int n = a.n;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gstride = nb * blockDim.x;
    double *partA = a.partials;
    double *partB = a.partials + nb;
    double *partC = a.partials + 2 * nb;
    double *partD = a.partials + 3 * nb;
    double ra, rb;
    const SpOp &A0 = M.lev[0].A;   // the solver's FP32 matrix (SELL-32)

    if (a.remove_mean) {
        double s = 0.0;
        for (int i = gtid; i < n; i += gstride) s += a.b[i];
        block_sum2(s, 0.0, sh, ra, rb);
        if (threadIdx.x == 0) partD[blockIdx.x] = ra;
        grid.sync();
        grid_sum2(partD, nullptr, nb, sh, ra, rb);
        if (threadIdx.x == 0) scal[0] = ra / (double)n;
        __syncthreads();
        const double mean = scal[0];
        for (int i = gtid; i < n; i += gstride) a.b[i] = a.b[i] - mean;
        grid.sync();
    }
    // r.z of the V-cycle just applied -> beta (thread 0 keeps rz)
    auto finish_rz = [&](double rz_part) {
        block_sum2(rz_part, 0.0, sh, ra, rb);
        if (threadIdx.x == 0) partA[blockIdx.x] = ra;
        grid.sync();
        grid_sum2(partA, nullptr, nb, sh, ra, rb);
        __syncthreads();
    };
    // solver scalars, kept by thread 0 in shared memory (no registers held
    // across the loop by the other threads)
    __shared__ double t_rz, t_tol2, t_rr, t_bb, t_rmax;
    __shared__ int t_it, t_status, t_updates;
    if (threadIdx.x == 0) {
        t_rz = t_tol2 = t_rr = t_bb = t_rmax = 0.0;
        t_it = 0; t_status = 1; t_updates = 0;
    }
    for (int pass = 0;; ++pass) {
        // true residual in FP64 into the FP32 recurrence
        double rr = 0.0, bb = 0.0;
        for (int i = gtid; i < n; i += gstride) {
            double s = 0.0;
            const int64_t base = a.slice_ptr[i >> 5] + (i & 31);
            const int w = a.slice_width[i >> 5];
#pragma unroll 4
            for (int k = 0; k < w; ++k) s = fma(__ldg(a.val + base + 32 * k), __ldcg(a.x + __ldg(a.col + base + 32 * k)), s);
            const double bi = a.b[i];
            const double ri = bi - s;
            a.r32[i] = (float)ri;
            rr = fma(ri, ri, rr);
            if (pass == 0) bb = fma(bi, bi, bb);
        }
        block_sum2(rr, bb, sh, ra, rb);
        if (threadIdx.x == 0) { partB[blockIdx.x] = ra; partC[blockIdx.x] = rb; }
        grid.sync();
        grid_sum2(partB, partC, nb, sh, ra, rb);
        if (threadIdx.x == 0) {
            t_rr = ra;
            if (pass == 0) {
                t_bb = rb;
                const double tol = fmax(a.rtol * sqrt(t_bb), a.atol);
                t_tol2 = tol * tol;
            } else {
                ++t_updates;
            }
            t_rmax = t_rr;
            if (t_rr <= t_tol2) { t_status = 0; scal[1] = 0.0; }
            else if (t_it >= a.max_iter) { t_status = 1; scal[1] = 0.0; }
            else scal[1] = 1.0;
        }
        __syncthreads();
        if (scal[1] == 0.0) break;
        // z = B r and r.z; beta = 0 on the first pass (p = z), else continue
        // the direction across the replacement
        finish_rz(vcycle(M, a.r32, a.z32, grid, gtid, gstride));
        if (threadIdx.x == 0) {
            scal[0] = pass > 0 ? ra / t_rz : 0.0;
            t_rz = ra;
        }
        __syncthreads();
        bool first = pass == 0;
        for (;;) {
            // A: p = z + beta p, Ap = A z + beta Ap, p.Ap
            const float beta = (float)scal[0];
            float pap32 = 0.0f;
            {
                const float *z = a.z32;
                float *p = a.p32, *Ap = a.Ap32;
                apply(A0, [=](int j) { return z[j]; },
                      [&](int i, float s) {
                          const float zi = z[i];
                          const float pi = first ? zi : fmaf(beta, p[i], zi);
                          const float api = first ? s : fmaf(beta, Ap[i], s);
                          p[i] = pi;
                          Ap[i] = api;
                          pap32 = fmaf(pi, api, pap32);
                      }, gtid, gstride);
            }
            first = false;
            block_sum2((double)pap32, 0.0, sh, ra, rb);
            if (threadIdx.x == 0) partA[blockIdx.x] = ra;
            grid.sync();
            grid_sum2(partA, nullptr, nb, sh, ra, rb);
            if (threadIdx.x == 0) {
                ++t_it;
                if (!(ra > 0.0)) { t_status = 2; scal[1] = 0.0; scal[0] = 0.0; }
                else { scal[0] = t_rz / ra; scal[1] = 1.0; }
            }
            __syncthreads();
            if (scal[1] == 0.0) break;
            // B: x, r update and ||r||^2 (rows of this thread as written in A)
            const double alpha = scal[0];
            const float alpha32 = (float)alpha;
            float rr32 = 0.0f;
            for (int i = gtid; i < n; i += 2 * gstride) {
                // two rows per pass, loads first
                const int i2 = i + gstride;
                const bool two = i2 < n;
                const double x1 = a.x[i];
                const float p1 = a.p32[i], q1 = a.Ap32[i], r1 = a.r32[i];
                const double x2 = two ? a.x[i2] : 0.0;
                const float p2 = two ? a.p32[i2] : 0.0f, q2 = two ? a.Ap32[i2] : 0.0f;
                const float r2 = two ? a.r32[i2] : 0.0f;
                const float n1 = fmaf(-alpha32, q1, r1), n2 = fmaf(-alpha32, q2, r2);
                a.x[i] = fma(alpha, (double)p1, x1);
                a.r32[i] = n1;
                rr32 = fmaf(n1, n1, rr32);
                if (two) {
                    a.x[i2] = fma(alpha, (double)p2, x2);
                    a.r32[i2] = n2;
                    rr32 = fmaf(n2, n2, rr32);
                }
            }
            block_sum2((double)rr32, 0.0, sh, ra, rb);
            if (threadIdx.x == 0) partC[blockIdx.x] = ra;
            grid.sync();
            grid_sum2(partC, nullptr, nb, sh, ra, rb);
            if (threadIdx.x == 0) {
                const double rr_rec = ra;
                scal[2] = (rr_rec <= 1e-6 * t_rmax || rr_rec <= t_tol2 || t_it >= a.max_iter) ? 1.0 : 0.0;
            }
            __syncthreads();
            if (scal[2] != 0.0) break;   // replace the residual (next pass)
            finish_rz(vcycle(M, a.r32, a.z32, grid, gtid, gstride));
            if (threadIdx.x == 0) { scal[0] = ra / t_rz; t_rz = ra; }
            __syncthreads();
        }
        if (scal[1] == 0.0) break;
        grid.sync();
    }
    if (a.remove_mean) {
        grid.sync();
        double s = 0.0;
        for (int i = gtid; i < n; i += gstride) s += a.x[i];
        block_sum2(s, 0.0, sh, ra, rb);
        if (threadIdx.x == 0) partB[blockIdx.x] = ra;
        grid.sync();
        grid_sum2(partB, nullptr, nb, sh, ra, rb);
        if (threadIdx.x == 0) scal[2] = ra / (double)n;
        __syncthreads();
        const double mean = scal[2];
        for (int i = gtid; i < n; i += gstride) a.x[i] = a.x[i] - mean;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *a.out_iter = t_it;
        *a.out_status = t_status;
        *a.out_rr = t_rr;
        *a.out_bb = t_bb;
        if (a.out_updates) *a.out_updates = t_updates;
    }
}

}  // namespace

int pcg_amg_grid_blocks() {
    static int g = 0;
    if (g == 0) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_amg, kPcgThreads, 0);
        if (per_sm < 1) per_sm = 1;
        if (per_sm > 2) per_sm = 2;
        g = per_sm * sm_count();
    }
    return g;
}

int launch_pcg_amg(const PcgArgs &a, const AmgDev &amg, cudaStream_t st) {
    int nb = pcg_amg_grid_blocks();
    const int need = (a.n + kPcgThreads - 1) / kPcgThreads;
    if (need < nb) nb = need < 1 ? 1 : need;
    PcgArgs arg = a;
    AmgDev m = amg;
    void *params[] = {&arg, &m};
    count_launches(1);
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_pcg_amg, dim3(nb), dim3(kPcgThreads), params, 0, st);
    return e == cudaSuccess ? 0 : (int)e;
}

}  // namespace pg
