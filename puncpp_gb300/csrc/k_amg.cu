// PCG preconditioned by one smoothed-aggregation AMG V-cycle per iteration,
// all in one cooperative launch.
//
// Krylov recurrence in FP32 with the solution, inner products and
// true-residual replacements in FP64 (as k_pcg_rel), stopping on the FP64
// true residual ||b - A x|| <= max(rtol ||b||, atol).  A replacement before
// the end of a solve (hierarchies of three or more levels) takes the true
// residual inside the iteration's own V-cycle; the one at the end is a new
// pass that restarts the cycle from the true residual.
//
// The V-cycle (one weighted-Jacobi sweep from zero before the coarse
// correction and one after, Galerkin coarse operators, dense coarsest
// inverse) is applied in the algebraically identical form
//     B_l b = W_l b + S_l B_{l+1} S_l^T b,   W = w D^-1 (2 I - A w D^-1),
//     S = (I - w D^-1 A) P,
// with the last restriction and the coarse solve in one product
// (G = C^-1 S^T) and the up-sweep of levels >= 1 collapsed into one product
// (U1 = [S_1 | S_1 S_2 | ...]): L + 2 grid-wide phases (L down, the
// up-sweep, the prolongation to level 0) for L >= 2 levels above the
// coarsest.  The product A z of the search direction update is
// folded into the next matrix phase (A p = A z + beta A p_old), r.z into the
// last cycle phase, and the x and r update of a CG step into the cycle's
// first phase (r - alpha Ap gathered on the fly, two residual buffers): with
// the phase of A p, an iteration is L + 3 grid barriers.  The smoothing products W_l b_l, needed
// only by the up-sweep, run in the down-sweep phases whose restrictions are
// small.
#include <cooperative_groups.h>
#include <cuda_fp16.h>
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
// epi(i, sum_j S_ij xv(j), pre(i)) for every row i of S, spread over the
// whole grid.  pre(i) loads the epilogue's own operands of row i before the
// row's gathers start.  A phase is a chain of dependent L2 round trips (row
// offsets -> column indices -> gathered values), so each thread keeps eight
// gathers in flight: SELL operators take one thread per row and four rows at
// a time, two entries of each per step; CSR operators g lanes per row, four
// rows per lane group at a time, reduced by warp shuffles (g <= 32), or the
// warps of one block per row, reduced through shared memory (g = 64..512).
// Every thread of the grid must call this (the CSR paths run the same number
// of rounds in all lanes so the shuffles are full-warp).
struct NoPre {
    __device__ __forceinline__ int operator()(int) const { return 0; }
};

constexpr int kRows = 4;   // rows per thread (SELL) or per lane group (CSR) at a time

// Column and value of stored entry o (b: the entry's slice or row base) in
// the operator's storage form.
// Read-only loads of operator entries that ask the L2 for the 256-byte
// segment around the address: the entries of the next step of a row (32 rows
// further in a SELL slice, the next lanes' share in CSR) arrive with this
// step's, so the next step's loads hit L2.
__device__ __forceinline__ uint16_t ld_nc_u16(const uint16_t *p) {
    uint16_t v;
    asm("ld.global.nc.L2::256B.u16 %0, [%1];" : "=h"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ int ld_nc_s32(const int32_t *p) {
    int v;
    asm("ld.global.nc.L2::256B.s32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ float ld_nc_f32(const float *p) {
    float v;
    asm("ld.global.nc.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}

template <bool C16, bool V16>
struct Entry {
    __device__ static __forceinline__ int col(const SpOp &S, int o, int b) {
        return C16 ? b + (int)ld_nc_u16(S.col16 + o) : ld_nc_s32(S.col + o);
    }
    __device__ static __forceinline__ float val(const SpOp &S, int o) {
        return V16 ? __half2float(__ushort_as_half(ld_nc_u16(S.val16 + o))) : ld_nc_f32(S.val + o);
    }
};

// This lane's share (entries lane, lane + g, ...) of row i of a CSR operator,
// four entries' loads issued before their products.
template <bool C16, bool V16, class XV>
__device__ __forceinline__ float csr_lane_sum(const SpOp &S, int i, int lane, int g, XV xv) {
    using E = Entry<C16, V16>;
    const int k0 = (int)__ldg(S.ptr + i);
    const int len = (int)__ldg(S.ptr + i + 1) - k0;
    const int b = C16 ? __ldg(S.cbase + i) : 0;
    float s0 = 0.0f, s1 = 0.0f;
    int k = lane;
    for (; k + 3 * g < len; k += 4 * g) {
        const int c0 = E::col(S, k0 + k, b), c1 = E::col(S, k0 + k + g, b);
        const int c2 = E::col(S, k0 + k + 2 * g, b), c3 = E::col(S, k0 + k + 3 * g, b);
        const float v0 = E::val(S, k0 + k), v1 = E::val(S, k0 + k + g);
        const float v2 = E::val(S, k0 + k + 2 * g), v3 = E::val(S, k0 + k + 3 * g);
        const float x0 = xv(c0), x1 = xv(c1), x2 = xv(c2), x3 = xv(c3);
        s0 = fmaf(v0, x0, s0);
        s1 = fmaf(v1, x1, s1);
        s0 = fmaf(v2, x2, s0);
        s1 = fmaf(v3, x3, s1);
    }
    for (; k < len; k += g) s0 = fmaf(E::val(S, k0 + k), xv(E::col(S, k0 + k, b)), s0);
    return s0 + s1;
}

constexpr int kWide = 8;   // SELL operators whose slices hold at most this many entries a row

template <bool C16, bool V16, class XV, class PRE, class EPI>
__device__ __forceinline__ void apply_t(const SpOp &S, XV xv, PRE pre, EPI epi, int t0, int ts) {
    using P = decltype(pre(0));
    using E = Entry<C16, V16>;
    const float vs = V16 ? S.vscale : 1.0f;
    if (S.g == 1 && S.wmax <= kWide) {
        // narrow SELL: every entry of two rows loaded at once, then every
        // gather, so a round costs three dependent trips (offsets, entries,
        // gathered values) instead of two per pair of entries; the sums run
        // in the same entry order as the general path below
        constexpr int R = 2;
        for (int i = t0; i < S.n; i += R * ts) {
            int off[R], wid[R], cb[R];
            P pv[R];
#pragma unroll
            for (int q = 0; q < R; ++q) {
                const int r = i + q * ts;
                const bool ok = r < S.n;
                off[q] = ok ? (int)__ldg(S.ptr + (r >> 5)) + (r & 31) : 0;
                wid[q] = ok ? __ldg(S.swidth + (r >> 5)) : 0;
                cb[q] = (ok && C16) ? __ldg(S.cbase + (r >> 5)) : 0;
                pv[q] = ok ? pre(r) : P{};
            }
            int c[R][kWide];
            float v[R][kWide];
#pragma unroll
            for (int q = 0; q < R; ++q)
#pragma unroll
                for (int k = 0; k < kWide; ++k) {
                    const bool ok = k < wid[q];
                    const int o = off[q] + 32 * k;
                    c[q][k] = ok ? E::col(S, o, cb[q]) : -1;
                    v[q][k] = ok ? E::val(S, o) : 0.0f;
                }
            float x[R][kWide];
#pragma unroll
            for (int q = 0; q < R; ++q)
#pragma unroll
                for (int k = 0; k < kWide; ++k) x[q][k] = c[q][k] >= 0 ? xv(c[q][k]) : 0.0f;
#pragma unroll
            for (int q = 0; q < R; ++q) {
                // the general path adds entries in pairs (a zero pair member
                // past an odd width included): the same operations here
                const int wpair = (wid[q] + 1) & ~1;
                float sum = 0.0f;
#pragma unroll
                for (int k = 0; k < kWide; ++k)
                    if (k < wpair) sum = fmaf(v[q][k], x[q][k], sum);
                if (i + q * ts < S.n) epi(i + q * ts, V16 ? sum * vs : sum, pv[q]);
            }
        }
    } else if (S.g == 1) {
        for (int i = t0; i < S.n; i += kRows * ts) {
            int off[kRows];   // operators hold fewer than 2^31 entries (checked at upload)
            int wid[kRows], cb[kRows];
            P pv[kRows];
            int w = 0;
#pragma unroll
            for (int q = 0; q < kRows; ++q) {
                const int r = i + q * ts;
                const bool ok = r < S.n;
                off[q] = ok ? (int)__ldg(S.ptr + (r >> 5)) + (r & 31) : 0;
                wid[q] = ok ? __ldg(S.swidth + (r >> 5)) : 0;
                cb[q] = (ok && C16) ? __ldg(S.cbase + (r >> 5)) : 0;
                pv[q] = ok ? pre(r) : P{};
                w = wid[q] > w ? wid[q] : w;
            }
            float sum[kRows];
#pragma unroll
            for (int q = 0; q < kRows; ++q) sum[q] = 0.0f;
            for (int k = 0; k < w; k += 2) {
                // entries k, k + 1 of the four rows (slice padding: value 0)
                int c[kRows][2];
                float v[kRows][2], x[kRows][2];
#pragma unroll
                for (int q = 0; q < kRows; ++q)
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const bool ok = k + e < wid[q];
                        const int o = off[q] + 32 * (k + e);
                        c[q][e] = ok ? E::col(S, o, cb[q]) : -1;
                        v[q][e] = ok ? E::val(S, o) : 0.0f;
                    }
#pragma unroll
                for (int q = 0; q < kRows; ++q)
#pragma unroll
                    for (int e = 0; e < 2; ++e) x[q][e] = c[q][e] >= 0 ? xv(c[q][e]) : 0.0f;
#pragma unroll
                for (int q = 0; q < kRows; ++q)
#pragma unroll
                    for (int e = 0; e < 2; ++e) sum[q] = fmaf(v[q][e], x[q][e], sum[q]);
            }
#pragma unroll
            for (int q = 0; q < kRows; ++q)
                if (i + q * ts < S.n) epi(i + q * ts, V16 ? sum[q] * vs : sum[q], pv[q]);
        }
    } else if (S.g <= 32) {
        const int g = S.g;
        const int lane = t0 & (g - 1);
        const int grp = t0 / g, ngrp = ts / g;
        const int rounds = (S.n + ngrp - 1) / ngrp;
        for (int t = 0; t < rounds; t += kRows) {
            // rounds t .. t + 3 together
            int off[kRows];
            int len[kRows], cb[kRows];
            P pv[kRows];
            int L = 0;
#pragma unroll
            for (int q = 0; q < kRows; ++q) {
                const int r = grp + (t + q) * ngrp;
                const bool ok = r < S.n;
                off[q] = ok ? (int)__ldg(S.ptr + r) : 0;
                len[q] = ok ? (int)__ldg(S.ptr + r + 1) - off[q] : 0;
                cb[q] = (ok && C16) ? __ldg(S.cbase + r) : 0;
                pv[q] = (ok && lane == 0) ? pre(r) : P{};
                L = len[q] > L ? len[q] : L;
            }
            float sum[kRows];
#pragma unroll
            for (int q = 0; q < kRows; ++q) sum[q] = 0.0f;
            for (int k = lane; k < L; k += 2 * g) {
                int c[kRows][2];
                float v[kRows][2], x[kRows][2];
#pragma unroll
                for (int q = 0; q < kRows; ++q)
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const int kk = k + e * g;
                        const bool ok = kk < len[q];
                        c[q][e] = ok ? E::col(S, off[q] + kk, cb[q]) : -1;
                        v[q][e] = ok ? E::val(S, off[q] + kk) : 0.0f;
                    }
#pragma unroll
                for (int q = 0; q < kRows; ++q)
#pragma unroll
                    for (int e = 0; e < 2; ++e) x[q][e] = c[q][e] >= 0 ? xv(c[q][e]) : 0.0f;
#pragma unroll
                for (int q = 0; q < kRows; ++q)
#pragma unroll
                    for (int e = 0; e < 2; ++e) sum[q] = fmaf(v[q][e], x[q][e], sum[q]);
            }
#pragma unroll
            for (int q = 0; q < kRows; ++q)
                for (int o = g >> 1; o > 0; o >>= 1) sum[q] += __shfl_xor_sync(0xffffffffu, sum[q], o);
            if (lane == 0) {
#pragma unroll
                for (int q = 0; q < kRows; ++q) {
                    const int r = grp + (t + q) * ngrp;
                    if (r < S.n) epi(r, V16 ? sum[q] * vs : sum[q], pv[q]);
                }
            }
        }
    } else {
        // g / 32 warps of one block per row; partial sums meet in shared memory
        __shared__ float red[kPcgThreads / 32];
        // (t0, ts) cover whole blocks: block t0 / blockDim of ts / blockDim
        const int g = S.g;
        const int per_block = blockDim.x / g;
        const int lane = threadIdx.x & (g - 1);
        const int grp = (t0 / (int)blockDim.x) * per_block + threadIdx.x / g;
        const int ngrp = (ts / (int)blockDim.x) * per_block;
        const int rounds = (S.n + ngrp - 1) / ngrp;
        for (int t = 0; t < rounds; ++t) {
            const int i = grp + t * ngrp;
            float s = i < S.n ? csr_lane_sum<C16, V16>(S, i, lane, g, xv) : 0.0f;
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
            __syncthreads();
            if (lane == 0 && i < S.n) {
                float tot = 0.0f;
                for (int w = 0; w < g / 32; ++w) tot += red[(threadIdx.x >> 5) + w];
                epi(i, V16 ? tot * vs : tot, pre(i));
            }
            __syncthreads();
        }
    }
}

// epi(i, (S xv)_i, pre(i)) over the whole grid.  V16: the operator's values
// are binary16 (fixed per operator at upload: the preconditioner's transfer
// and coarse operators; A_0, G and the coarsest inverse keep FP32, which the
// set-up checks); the column width is chosen by a uniform branch.
template <bool V16, class XV, class PRE, class EPI>
__device__ __forceinline__ void apply(const SpOp &S, XV xv, PRE pre, EPI epi, int t0, int ts) {
    if (S.col16) apply_t<true, V16>(S, xv, pre, epi, t0, ts);
    else apply_t<false, V16>(S, xv, pre, epi, t0, ts);
}

// Blocks that take one pass over S (kRows rows per thread or lane group,
// one row per lane group of the block path).
__device__ __forceinline__ int pass_blocks(const SpOp &S) {
    const int bd = blockDim.x;
    if (S.g > 32) {
        const int per_block = bd / S.g;
        return (S.n + per_block - 1) / per_block;
    }
    const int64_t threads = (int64_t)((S.n + kRows - 1) / kRows) * S.g;
    return (int)((threads + bd - 1) / bd);
}

// Independent products of one grid phase on disjoint ranges of blocks, so
// that their latency chains run side by side instead of one after another:
// when the k <= 4 products' one-pass needs n0..n3 fit in the grid, each gets
// its need (the largest also the spare blocks).  Returns this block's product
// and range, or -1 (run them all, one after another, on the whole grid) when
// they do not fit: a product squeezed into fewer blocks would take a second
// pass and lengthen its chain.
__device__ __forceinline__ int split_blocks(int k, int n0, int n1, int n2, int n3, int nb, int &lo, int &hi) {
    const int need[4] = {n0 > 0 ? n0 : 1, n1 > 0 ? n1 : 1, n2 > 0 ? n2 : 1, n3 > 0 ? n3 : 1};
    int tot = 0, big = 0, bigv = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (i < k) {
            tot += need[i];
            if (need[i] > bigv) { bigv = need[i]; big = i; }
        }
    if (k < 2 || tot > nb) return -1;
    int mine = -1, b = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (i < k) {
            const int share = need[i] + (i == big ? nb - tot : 0);
            if ((int)blockIdx.x >= b && (int)blockIdx.x < b + share) { mine = i; lo = b; hi = b + share; }
            b += share;
        }
    return mine;
}

// The residual as phase 0 of a V-cycle reads it: right after a CG step the
// step's update r - alpha Ap is formed on the fly from the previous residual
// (the same FP32 expression the rows' owners store), so the update needs no
// phase of its own.
template <bool kMerge>
struct ResGather {
    const float *r, *Ap;
    float alpha;
    __device__ __forceinline__ float operator()(int j) const { return kMerge ? fmaf(-alpha, Ap[j], r[j]) : r[j]; }
};

// t = W x for level Lv: W = w D^-1 (2 I - A w D^-1), xg(j) the input vector.
template <bool V16, class XG>
__device__ __forceinline__ void smooth(const AmgLevelDev &Lv, XG xg, float *t, int t0, int ts) {
    const float om = Lv.omega;
    const float *dinv = Lv.dinv;
    apply<V16>(Lv.A, [=](int j) { return om * __ldg(dinv + j) * xg(j); },
          [=](int i) { return make_float2(__ldg(dinv + i), xg(i)); },
          [=](int i, float s, float2 dx) { t[i] = om * dx.x * (2.0f * dx.y - s); }, t0, ts);
}

// Phase 0 of z = B r: the first restriction b_1 = S_0^T r (L >= 2), or
// y_L = G r and t_0 = W_0 r (L == 1), or z = C^-1 r (L == 0, returning this
// thread's share of r.z).  With kMerge, the CG step's x += alpha p and
// r_new = r - alpha Ap of this thread's rows (r_new into rn) and ||r_new||^2
// (into rr) run in the same phase.
template <bool kMerge>
__device__ double vcycle_phase0(const AmgDev &M, const PcgArgs &a, const float *r, float *rn, double alpha,
                                float *z, float &rr, int t0, int ts) {
    const int n = a.n;
    const float alpha32 = (float)alpha;
    const ResGather<kMerge> gr{r, a.Ap32, alpha32};
    if (kMerge) {
        float acc = 0.0f;
        for (int i = t0; i < n; i += 2 * ts) {
            // two rows per pass, loads first
            const int i2 = i + ts;
            const bool two = i2 < n;
            const double x1 = a.x[i];
            const float p1 = a.p32[i], q1 = a.Ap32[i], r1 = r[i];
            const double x2 = two ? a.x[i2] : 0.0;
            const float p2 = two ? a.p32[i2] : 0.0f, q2 = two ? a.Ap32[i2] : 0.0f;
            const float r2 = two ? r[i2] : 0.0f;
            const float n1 = fmaf(-alpha32, q1, r1), n2 = fmaf(-alpha32, q2, r2);
            a.x[i] = fma(alpha, (double)p1, x1);
            rn[i] = n1;
            acc = fmaf(n1, n1, acc);
            if (two) {
                a.x[i2] = fma(alpha, (double)p2, x2);
                rn[i2] = n2;
                acc = fmaf(n2, n2, acc);
            }
        }
        rr = acc;
    }
    const int L = M.nlev - 1;
    double rz = 0.0;
    if (L == 0) {
        apply<false>(M.cinv, gr, [=](int i) { return gr(i); },
              [&](int i, float s, float ri) { z[i] = s; rz = fma((double)s, (double)ri, rz); }, t0, ts);
    } else if (L == 1) {
        float *yL = M.yL;
        apply<false>(M.G, gr, NoPre{}, [=](int i, float s, int) { yL[i] = s; }, t0, ts);
        smooth<false>(M.lev[0], gr, M.lev[0].t, t0, ts);
    } else {
        float *b1 = M.lev[1].b;
        apply<true>(M.lev[0].ST, gr, NoPre{}, [=](int i, float s, int) { b1[i] = s; }, t0, ts);
    }
    return rz;
}

// The FP64 true residual b - A x of this thread's rows (A the solver's FP64
// SELL matrix; x read through L2, it is written inside the kernel) into r in
// FP32; returns this thread's share of ||b - A x||^2 and, with want_bb, adds
// its share of ||b||^2 to bb.
__device__ __forceinline__ double true_residual(const PcgArgs &a, float *r, bool want_bb, double &bb, int t0,
                                                int ts) {
    double rr = 0.0;
    for (int i = t0; i < a.n; i += ts) {
        double s = 0.0;
        const int64_t base = a.slice_ptr[i >> 5] + (i & 31);
        const int w = a.slice_width[i >> 5];
#pragma unroll 4
        for (int k = 0; k < w; ++k) s = fma(__ldg(a.val + base + 32 * k), __ldcg(a.x + __ldg(a.col + base + 32 * k)), s);
        const double bi = a.b[i];
        const double ri = bi - s;
        r[i] = (float)ri;
        rr = fma(ri, ri, rr);
        if (want_bb) bb = fma(bi, bi, bb);
    }
    return rr;
}

// Phases 1 .. of z = B r after phase 0 (L >= 1, r the current residual,
// complete): down-sweep phases l = 1 .. L-1 (restriction or, at l = L-1,
// G; smoothing t_l of levels l >= 2 into the stack; t_0 = W_0 r in phase 1
// and t_1 = W_1 b_1 in phase L-1, where the restrictions leave the grid
// idle), the collapsed up-sweep y_1 = t_1 + U1 [t_2 .. t_{L-1}, y_L]
// (L >= 2), then z = t_0 + S_0 y_1; returns this thread's share of r.z.
//
// With rt (L >= 2): a residual replacement that keeps this cycle.  The FP64
// true residual of the current x goes to rt (FP32) in the coarse phase l =
// L-1, where the products are small, with its block partials of ||b - A x||^2
// in part_rt; the returned r.z is taken against rt.  z = B r of the recurrence
// residual r then stands for B rt: they differ by the recurrence's drift.
__device__ __forceinline__ double vcycle_rest(const AmgDev &M, const float *r, float *z, cg::grid_group &grid,
                                              int t0, int ts, const PcgArgs &a, float *rt, double *part_rt,
                                              double *sh) {
    const int L = M.nlev - 1;
    for (int l = 1; l < L; ++l) {
        const float *b = M.lev[l].b;
        const auto gb = [=](int j) { return b[j]; };
        // this phase's independent products, each on its own blocks
        const SpOp &R = l < L - 1 ? M.lev[l].ST : M.G;
        const int nR = pass_blocks(R);
        const int nS = l >= 2 ? pass_blocks(M.lev[l].A) : 0;
        const int n0 = l == 1 ? pass_blocks(M.lev[0].A) : 0;
        const int n1 = l == L - 1 ? pass_blocks(M.lev[1].A) : 0;
        // product order: R, then W_l (l >= 2), W_0 (l == 1), W_1 (l == L-1)
        int need[4] = {nR, 0, 0, 0}, k = 1;
        if (l >= 2) need[k++] = nS;
        if (l == 1) need[k++] = n0;
        if (l == L - 1) need[k++] = n1;
        int lo = 0, hi = 0;
        const int my = split_blocks(k, need[0], k > 1 ? need[1] : 0, k > 2 ? need[2] : 0, k > 3 ? need[3] : 0,
                                    (int)gridDim.x, lo, hi);
        int idx = 0, pt0 = t0, pts = ts;
        const auto mine = [&](int q) {
            if (my < 0) { pt0 = t0; pts = ts; return true; }
            if (q != my) return false;
            pt0 = ((int)blockIdx.x - lo) * (int)blockDim.x + (int)threadIdx.x;
            pts = (hi - lo) * (int)blockDim.x;
            return true;
        };
        if (mine(idx++)) {
            if (l < L - 1) {
                float *bn = M.lev[l + 1].b;
                apply<true>(R, gb, NoPre{}, [=](int i, float s, int) { bn[i] = s; }, pt0, pts);
            } else {
                float *yL = M.yL;
                apply<false>(R, gb, NoPre{}, [=](int i, float s, int) { yL[i] = s; }, pt0, pts);
            }
        }
        if (l >= 2 && mine(idx++)) smooth<true>(M.lev[l], gb, M.lev[l].t, pt0, pts);
        if (l == 1 && mine(idx++)) smooth<false>(M.lev[0], [=](int j) { return r[j]; }, M.lev[0].t, pt0, pts);
        if (l == L - 1 && mine(idx++)) {
            const float *b1 = M.lev[1].b;
            smooth<true>(M.lev[1], [=](int j) { return b1[j]; }, M.lev[1].t, pt0, pts);
        }
        if (rt && l == L - 1) {
            double unused = 0.0, ra, rb;
            const double rr = true_residual(a, rt, false, unused, t0, ts);
            block_sum2(rr, 0.0, sh, ra, rb);
            if (threadIdx.x == 0) part_rt[blockIdx.x] = ra;
        }
        grid.sync();
    }
    const float *yup = M.yL;
    if (L >= 2) {
        const float *t1 = M.lev[1].t, *st = M.stack;
        float *y1 = M.y1;
        apply<true>(M.U1, [=](int j) { return st[j]; }, [=](int i) { return t1[i]; },
              [=](int i, float s, float ti) { y1[i] = ti + s; }, t0, ts);
        grid.sync();
        yup = M.y1;
    }
    const float *tz = M.lev[0].t;
    const float *rzv = rt ? rt : r;
    double rz = 0.0;
    apply<true>(M.S0, [=](int j) { return yup[j]; }, [=](int i) { return make_float2(tz[i], rzv[i]); },
          [&](int i, float s, float2 tr) {
              const float zi = tr.x + s;
              z[i] = zi;
              rz = fma((double)zi, (double)tr.y, rz);
          }, t0, ts);
    return rz;
}

// Block partials of the grid reductions: p.Ap in A, ||r||^2 of the merged
// update in B, r.z in C, the pass start's (||r||^2, ||b||^2) in (B, D).  A
// buffer is written again only after at least one grid barrier has passed
// since every block read it.
__global__ void __launch_bounds__(kPcgThreads, 2) k_pcg_amg(PcgArgs a, AmgDev M) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[2 * kPcgThreads + 16];
    __shared__ double scal[5];
    const int nb = gridDim.x;
    const int n = a.n;
    const int L = M.nlev - 1;
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
    // solver scalars, kept by thread 0 in shared memory (no registers held
    // across the loop by the other threads)
    __shared__ double t_rz, t_tol2, t_rr, t_bb, t_rmax;
    __shared__ int t_it, t_status, t_updates;
    if (threadIdx.x == 0) {
        t_rz = t_tol2 = t_rr = t_bb = t_rmax = 0.0;
        t_it = 0; t_status = 1; t_updates = 0;
    }
    // the two residual buffers: r is the current one
    float *r = a.r32, *rn = M.r_alt;
    for (int pass = 0;; ++pass) {
        // true residual in FP64 into the FP32 recurrence
        double bb = 0.0;
        const double rr = true_residual(a, r, pass == 0, bb, gtid, gstride);
        block_sum2(rr, bb, sh, ra, rb);
        if (threadIdx.x == 0) { partB[blockIdx.x] = ra; partD[blockIdx.x] = rb; }
        grid.sync();
        grid_sum2(partB, partD, nb, sh, ra, rb);
        if (threadIdx.x == 0) {
            // between replacements the FP32 recurrence's ||r||^2 falls by 1e6;
            // a true residual that fell by less than 100 (10 in norm) means
            // the recurrence has left the true residual at its attainable
            // accuracy above the requested tolerance: stop (status 3)
            // instead of iterating on
            const bool stalled = pass > 0 && ra > 1e-2 * t_rr;
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
            else if (stalled) { t_status = 3; scal[1] = 0.0; }
            else scal[1] = 1.0;
        }
        __syncthreads();
        if (scal[1] == 0.0) break;
        // z = B r and r.z; beta = 0 on the first pass (p = z), else continue
        // the direction across the replacement
        {
            float unused = 0.0f;
            const double rz0 = vcycle_phase0<false>(M, a, r, rn, 0.0, a.z32, unused, gtid, gstride);
            if (L == 0) {
                block_sum2(rz0, 0.0, sh, ra, rb);
                if (threadIdx.x == 0) partC[blockIdx.x] = ra;
            }
            grid.sync();
            if (L >= 1) {
                const double rzp = vcycle_rest(M, r, a.z32, grid, gtid, gstride, a, nullptr, nullptr, sh);
                block_sum2(rzp, 0.0, sh, ra, rb);
                if (threadIdx.x == 0) partC[blockIdx.x] = ra;
                grid.sync();
            }
            grid_sum2(partC, nullptr, nb, sh, ra, rb);
            if (threadIdx.x == 0) {
                scal[0] = pass > 0 ? ra / t_rz : 0.0;
                t_rz = ra;
            }
            __syncthreads();
        }
        bool first = pass == 0;
        for (;;) {
            // A: p = z + beta p, Ap = A z + beta Ap, p.Ap
            const float beta = (float)scal[0];
            float pap32 = 0.0f;
            {
                const float *z = a.z32;
                float *p = a.p32, *Ap = a.Ap32;
                apply<false>(A0, [=](int j) { return z[j]; }, [=](int i) { return make_float3(z[i], p[i], Ap[i]); },
                      [&](int i, float s, float3 zpa) {
                          const float pi = first ? zpa.x : fmaf(beta, zpa.y, zpa.x);
                          const float api = first ? s : fmaf(beta, zpa.z, s);
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
            // B + phase 0 of the next cycle: x += alpha p, r_new = r - alpha Ap
            // into rn with ||r_new||^2, and phase 0 on r_new
            float rr32 = 0.0f;
            const double rz0 = vcycle_phase0<true>(M, a, r, rn, scal[0], a.z32, rr32, gtid, gstride);
            block_sum2((double)rr32, rz0, sh, ra, rb);
            if (threadIdx.x == 0) { partB[blockIdx.x] = ra; if (L == 0) partC[blockIdx.x] = rb; }
            grid.sync();
            {
                float *t = r; r = rn; rn = t;
            }
            grid_sum2(partB, L == 0 ? partC : nullptr, nb, sh, ra, rb);
            if (threadIdx.x == 0) {
                // replacement: at the end (tolerance or cap) by a new pass;
                // between (the recurrence fell by 1e6 in ||r||^2) inside this
                // cycle when L >= 2
                const double rr_rec = ra;
                const bool last = rr_rec <= t_tol2 || t_it >= a.max_iter;
                scal[2] = (last || (rr_rec <= 1e-6 * t_rmax && L < 2)) ? 1.0 : 0.0;
                scal[4] = (!last && rr_rec <= 1e-6 * t_rmax && L >= 2) ? 1.0 : 0.0;
                scal[3] = rb;
            }
            __syncthreads();
            if (scal[2] != 0.0) break;   // replace the residual (next pass)
            const bool keep = scal[4] != 0.0;
            double rz = scal[3];
            if (L >= 1) {
                const double rzp = vcycle_rest(M, r, a.z32, grid, gtid, gstride, a, keep ? rn : nullptr, partD, sh);
                block_sum2(rzp, 0.0, sh, ra, rb);
                if (threadIdx.x == 0) partC[blockIdx.x] = ra;
                grid.sync();
                grid_sum2(partC, keep ? partD : nullptr, nb, sh, ra, rb);
                rz = ra;
            }
            if (threadIdx.x == 0) {
                scal[1] = 1.0;
                if (keep) {
                    // the true residual replaces the recurrence's (as at a
                    // pass start, with the same stall test)
                    const bool stalled = rb > 1e-2 * t_rr;
                    t_rr = rb;
                    t_rmax = rb;
                    ++t_updates;
                    if (t_rr <= t_tol2) { t_status = 0; scal[1] = 0.0; }
                    else if (stalled) { t_status = 3; scal[1] = 0.0; }
                }
                scal[0] = rz / t_rz;
                t_rz = rz;
            }
            __syncthreads();
            if (keep) {
                float *t = r; r = rn; rn = t;
            }
            if (scal[1] == 0.0) break;
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
