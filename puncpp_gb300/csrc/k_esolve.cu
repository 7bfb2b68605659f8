// CG1 electric field: ESolver (punc/src/efield.cpp:41-75, punc/ufl/EField3D.ufl)
// solves the L2 projection of -grad(phi) onto continuous piecewise-linear
// vector fields,  M E_c = b_c  for the three components, with M the consistent
// P1 mass matrix and b_c,d = integral of (-d phi/dx_c) lambda_d = sum over the
// cells T of dof d of (vol_T / 4) (-grad phi_T)_c.
//
// The rhs is gathered per dof over its cells in ascending cell order
// (deterministic).  The three systems are solved together by Jacobi-
// preconditioned CG in one cooperative launch: one pass over a row of M serves
// the three components, and the update of A p is folded into the product phase
// (A p = A z + beta A p_old), so an iteration is two grid barriers.  D^-1 M has
// its spectrum in [1/2, 5/2] on any P1 tetrahedral mesh (the element mass
// matrices (vol/20)(I + 1 1^T) scaled by their diagonal), so CG needs ~25
// iterations for 1e-12.  Arithmetic in T (double for the FP64 form, float for
// the mixed form); reductions in FP64.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "pg_device.cuh"
#include "pg_reduce.cuh"

namespace cg = cooperative_groups;

namespace pg {

namespace {

constexpr int kThreads = 256;

template <typename T>
__global__ void k_esolve_rhs(int32_t ndof, const int64_t *__restrict__ adj_ptr, const int32_t *__restrict__ adj_cell,
                             const double *__restrict__ vol, const double *__restrict__ E, T *__restrict__ b) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= ndof) return;
    double bx = 0.0, by = 0.0, bz = 0.0;
    for (int64_t k = adj_ptr[d]; k < adj_ptr[d + 1]; ++k) {
        const int c = adj_cell[k];
        const double w = 0.25 * vol[c];
        const double2 e01 = __ldg(reinterpret_cast<const double2 *>(E) + 2 * (size_t)c);
        const double e2 = __ldg(E + 4 * (size_t)c + 2);
        bx = bx + w * e01.x;
        by = by + w * e01.y;
        bz = bz + w * e2;
    }
    b[d] = (T)bx;
    b[ndof + d] = (T)by;
    b[2 * ndof + d] = (T)bz;
}

// Sum over the block of N per-thread values; valid in every thread after the
// call (sh: at least 17 * N doubles).
template <int N>
__device__ __forceinline__ void block_sum_n(const double (&v)[N], double *sh, double (&out)[N]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        double a = v[k];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) sh[w * N + k] = a;
    }
    __syncthreads();
    for (int k = w; k < N; k += nw) {
        double a = lane < nw ? sh[lane * N + k] : 0.0;
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) sh[16 * N + k] = a;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) out[k] = sh[16 * N + k];
    __syncthreads();
}

// Sum of per-block partials part[k * nb + b] over b, for k < N; valid in every
// thread (one warp per component).
template <int N>
__device__ __forceinline__ void grid_sum_n(const double *part, int nb, double *sh, double (&out)[N]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = w; k < N; k += nw) {
        double a = 0.0;
        for (int b = lane; b < nb; b += 32) a += part[k * nb + b];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) sh[k] = a;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) out[k] = sh[k];
    __syncthreads();
}

template <typename T>
struct Cg3Args {
    int32_t n;
    const int32_t *row, *col;
    const T *val, *dinv;
    const T *b;                   // [3][n]
    T *x, *r, *z, *p, *Ap;        // [3][n]
    double *partials;             // [12][grid]
    double rtol, atol;
    int32_t max_iter;
    int32_t *out_iter, *out_status;
    double *out_rr, *out_bb;      // [3] each
};

// Partials: region A (3 x grid) for p.Ap, region B (9 x grid) for the other
// sums; alternating regions lets a block write its next partials while slower
// blocks still read the previous ones, so an iteration needs two barriers.
template <typename T>
__global__ void __launch_bounds__(kThreads, 3) k_mass_cg3(Cg3Args<T> a) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[17 * 9];
    const int nb = gridDim.x, n = a.n;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gs = nb * blockDim.x;
    double *partA = a.partials, *partB = a.partials + 3 * nb;
    const T *val = a.val;
    // r = b - M x, z = D^-1 r; ||b||^2, r.z, ||r||^2
    double rz[3], bb[3], rr[3], tol2[3];
    {
        double loc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = gtid; i < n; i += gs) {
            T s0 = 0, s1 = 0, s2 = 0;
            for (int k = a.row[i]; k < a.row[i + 1]; ++k) {
                const int j = a.col[k];
                const T v = val[k];
                s0 += v * a.x[j];
                s1 += v * a.x[n + j];
                s2 += v * a.x[2 * n + j];
            }
            const T s[3] = {s0, s1, s2};
            const T di = a.dinv[i];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T bi = a.b[c * n + i];
                const T ri = bi - s[c];
                const T zi = di * ri;
                a.r[c * n + i] = ri;
                a.z[c * n + i] = zi;
                loc[c] += (double)bi * (double)bi;
                loc[3 + c] += (double)ri * (double)zi;
                loc[6 + c] += (double)ri * (double)ri;
            }
        }
        double out[9];
        block_sum_n<9>(loc, sh, out);
#pragma unroll
        for (int k = 0; k < 9; ++k)
            if (threadIdx.x == k) partB[k * nb + blockIdx.x] = out[k];
        grid.sync();
        grid_sum_n<9>(partB, nb, sh, out);
        for (int c = 0; c < 3; ++c) {
            bb[c] = out[c];
            rz[c] = out[3 + c];
            rr[c] = out[6 + c];
            const double tol = fmax(a.rtol * sqrt(bb[c]), a.atol);
            tol2[c] = tol * tol;
        }
    }
    int it = 0;
    bool done = rr[0] <= tol2[0] && rr[1] <= tol2[1] && rr[2] <= tol2[2];
    double beta[3] = {0.0, 0.0, 0.0};
    bool first = true;
    while (!done && it < a.max_iter) {
        // A: p = z + beta p, Ap = M z + beta Ap, p.Ap
        double pap[3] = {0.0, 0.0, 0.0};
        for (int i = gtid; i < n; i += gs) {
            T s0 = 0, s1 = 0, s2 = 0;
            for (int k = a.row[i]; k < a.row[i + 1]; ++k) {
                const int j = a.col[k];
                const T v = val[k];
                s0 += v * a.z[j];
                s1 += v * a.z[n + j];
                s2 += v * a.z[2 * n + j];
            }
            const T s[3] = {s0, s1, s2};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T zi = a.z[c * n + i];
                const T pi = first ? zi : zi + (T)beta[c] * a.p[c * n + i];
                const T api = first ? s[c] : s[c] + (T)beta[c] * a.Ap[c * n + i];
                a.p[c * n + i] = pi;
                a.Ap[c * n + i] = api;
                pap[c] += (double)pi * (double)api;
            }
        }
        first = false;
        double alpha[3];
        {
            double out[3];
            block_sum_n<3>(pap, sh, out);
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if (threadIdx.x == k) partA[k * nb + blockIdx.x] = out[k];
            grid.sync();
            grid_sum_n<3>(partA, nb, sh, out);
            for (int c = 0; c < 3; ++c) alpha[c] = (rr[c] > tol2[c] && out[c] > 0.0) ? rz[c] / out[c] : 0.0;
        }
        ++it;
        // B: x += alpha p, r -= alpha Ap, z = D^-1 r; r.z, ||r||^2 (rows of this
        // thread, written in A)
        double loc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = gtid; i < n; i += gs) {
            const T di = a.dinv[i];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T al = (T)alpha[c];
                a.x[c * n + i] += al * a.p[c * n + i];
                const T ri = a.r[c * n + i] - al * a.Ap[c * n + i];
                const T zi = di * ri;
                a.r[c * n + i] = ri;
                a.z[c * n + i] = zi;
                loc[c] += (double)ri * (double)zi;
                loc[3 + c] += (double)ri * (double)ri;
            }
        }
        {
            double out[9];
            block_sum_n<9>(loc, sh, out);
    #pragma unroll
        for (int k = 0; k < 9; ++k)
            if (threadIdx.x == k) partB[k * nb + blockIdx.x] = out[k];
            grid.sync();
            grid_sum_n<9>(partB, nb, sh, out);
            for (int c = 0; c < 3; ++c) {
                beta[c] = rz[c] > 0.0 ? out[c] / rz[c] : 0.0;
                rz[c] = out[c];
                if (rr[c] > tol2[c]) rr[c] = out[3 + c];
            }
        }
        done = rr[0] <= tol2[0] && rr[1] <= tol2[1] && rr[2] <= tol2[2];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *a.out_iter = it;
        *a.out_status = done ? 0 : 1;
        for (int c = 0; c < 3; ++c) { a.out_rr[c] = rr[c]; a.out_bb[c] = bb[c]; }
    }
}

template <typename T>
__global__ void k_pack_ev(int32_t n, const T *__restrict__ x, double e0x, double e0y, double e0z,
                          double *__restrict__ ev, float *__restrict__ evf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double ex = (double)x[i] + e0x, ey = (double)x[n + i] + e0y, ez = (double)x[2 * n + i] + e0z;
    if (ev) {
        reinterpret_cast<double2 *>(ev)[2 * (size_t)i] = make_double2(ex, ey);
        reinterpret_cast<double2 *>(ev)[2 * (size_t)i + 1] = make_double2(ez, 0.0);
    }
    if (evf) reinterpret_cast<float4 *>(evf)[i] = make_float4((float)ex, (float)ey, (float)ez, 0.0f);
}

template <typename T>
int grid_blocks() {
    static int g = 0;
    if (g == 0) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mass_cg3<T>, kThreads, 0);
        if (per_sm < 1) per_sm = 1;
        if (per_sm > 3) per_sm = 3;
        g = per_sm * sm_count();
    }
    return g;
}

}  // namespace

int esolve_grid_blocks() { return grid_blocks<double>() > grid_blocks<float>() ? grid_blocks<double>() : grid_blocks<float>(); }

int launch_esolve(const EsolveArgs &e, cudaStream_t st) {
    const int n = e.n;
    if (n <= 0) return 0;
    const int blocks = (n + kThreads - 1) / kThreads;
    count_launches(3);
    if (e.fp32) {
        k_esolve_rhs<float><<<blocks, kThreads, 0, st>>>(n, e.adj_ptr, e.adj_cell, e.vol, e.E_cell, e.b32);
        Cg3Args<float> a{n, e.row, e.col, e.val32, e.dinv32, e.b32, e.x32, e.r32, e.z32, e.p32, e.Ap32,
                         e.partials, e.rtol, e.atol, e.max_iter, e.out_iter, e.out_status, e.out_rr, e.out_bb};
        int nb = grid_blocks<float>();
        if (blocks < nb) nb = blocks;
        void *params[] = {&a};
        cudaError_t err = cudaLaunchCooperativeKernel((const void *)k_mass_cg3<float>, dim3(nb), dim3(kThreads), params,
                                                      0, st);
        if (err != cudaSuccess) return (int)err;
        k_pack_ev<float><<<blocks, kThreads, 0, st>>>(n, e.x32, e.E0[0], e.E0[1], e.E0[2], e.ev, e.evf);
    } else {
        k_esolve_rhs<double><<<blocks, kThreads, 0, st>>>(n, e.adj_ptr, e.adj_cell, e.vol, e.E_cell, e.b);
        Cg3Args<double> a{n, e.row, e.col, e.val, e.dinv, e.b, e.x, e.r, e.z, e.p, e.Ap,
                          e.partials, e.rtol, e.atol, e.max_iter, e.out_iter, e.out_status, e.out_rr, e.out_bb};
        int nb = grid_blocks<double>();
        if (blocks < nb) nb = blocks;
        void *params[] = {&a};
        cudaError_t err = cudaLaunchCooperativeKernel((const void *)k_mass_cg3<double>, dim3(nb), dim3(kThreads),
                                                      params, 0, st);
        if (err != cudaSuccess) return (int)err;
        k_pack_ev<double><<<blocks, kThreads, 0, st>>>(n, e.x, e.E0[0], e.E0[1], e.E0[2], e.ev, e.evf);
    }
    return (int)cudaGetLastError();
}

void launch_pack_ev64(int32_t n, const double *x3, const double E0[3], double *ev, float *evf, cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1);
    k_pack_ev<double><<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(n, x3, E0[0], E0[1], E0[2], ev, evf);
}

}  // namespace pg
