// Jacobi-preconditioned CG on a caller's CSR matrix that allocates nothing.
//
// Some callers cannot allocate device memory: a host application that hands
// out all GPU memory at start-up and forbids later allocations, a solver
// embedded in another framework's memory pool, or a real-time loop that must
// not risk an allocation failure or the device-wide synchronisation cudaMalloc
// and cudaFree can cause.  For them this entry point keeps its work vectors
// in a file-scope static __device__ array of fixed size instead of buffers
// from cudaMalloc; the caller passes only the matrix, the right-hand side and
// the solution, all in device memory it already owns.
//
// Limits and sharing:
//   * at most kMaxRows rows (2^19 = 524,288): the array holds five vectors of
//     that length plus per-block partial sums, about 20 MB, which every GPU
//     that loads the library keeps until the process exits;
//   * every call uses the same array, so calls that overlap on the GPU (for
//     example on two streams) race; the array keeps the last call's contents,
//     and each call initialises every value it reads before reading it;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, which may load the module) and the kernel's
//     occupancy.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "pg_device.cuh"
#include "pg_internal.h"

namespace cg = cooperative_groups;

namespace pg {

namespace {

constexpr int kNaThreads = 512;
constexpr int64_t kMaxRows = int64_t(1) << 19;
constexpr int kMaxBlocks = 2048;
// r, z, p, Ap, D^-1 | partials [4][kMaxBlocks] | iteration, status, ||r||^2, ||b||^2
constexpr size_t kScratchDoubles = 5 * (size_t)kMaxRows + 4 * (size_t)kMaxBlocks + 8;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

struct NoAllocArgs {
    int32_t n;
    const int32_t *rowptr;
    const int32_t *col;
    const double *val;
    const double *b;
    double *x;
    double rtol, atol;
    int32_t max_iter;
    double *scratch;     // device address of g_noalloc_scratch
};

// Block sum of two values through shared memory (warps 0-3 add), valid in thread 0.
__device__ __forceinline__ void na_block_sum2(double a, double b, double *sh, double &ra, double &rb) {
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    sh[t] = a;
    sh[kNaThreads + t] = b;
    __syncthreads();
    if (w < 4) {
        const int q = kNaThreads / 4;
        double sa = 0.0, sb = 0.0;
        for (int k = lane; k < q; k += 32) { sa += sh[w * q + k]; sb += sh[kNaThreads + w * q + k]; }
        for (int o = 16; o > 0; o >>= 1) {
            sa += __shfl_down_sync(0xffffffffu, sa, o);
            sb += __shfl_down_sync(0xffffffffu, sb, o);
        }
        if (lane == 0) { sh[2 * kNaThreads + w] = sa; sh[2 * kNaThreads + 4 + w] = sb; }
    }
    __syncthreads();
    if (t == 0) {
        const double *r = sh + 2 * kNaThreads;
        ra = (r[0] + r[1]) + (r[2] + r[3]);
        rb = (r[4] + r[5]) + (r[6] + r[7]);
    }
}

// Sum of per-block partials (same order in every block), valid in thread 0.
// Ends with a block barrier, so that the next call's warp sums cannot
// overwrite the shared slots before thread 0 has read them.
__device__ __forceinline__ void na_grid_sum2(const double *pa, const double *pb, int nb, double *sh, double &ra,
                                             double &rb) {
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    if (w < 4) {
        double sa = 0.0, sb = 0.0;
        for (int k = w * 32 + lane; k < nb; k += 128) { sa += __ldcg(pa + k); sb += __ldcg(pb + k); }
        for (int o = 16; o > 0; o >>= 1) {
            sa += __shfl_down_sync(0xffffffffu, sa, o);
            sb += __shfl_down_sync(0xffffffffu, sb, o);
        }
        if (lane == 0) { sh[2 * kNaThreads + 8 + w] = sa; sh[2 * kNaThreads + 12 + w] = sb; }
    }
    __syncthreads();
    if (t == 0) {
        const double *r = sh + 2 * kNaThreads + 8;
        ra = (r[0] + r[1]) + (r[2] + r[3]);
        rb = (r[4] + r[5]) + (r[6] + r[7]);
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kNaThreads, 2) k_pcg_csr_noalloc(NoAllocArgs a) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[2 * kNaThreads + 16];
    __shared__ double scal[2];
    const int nb = gridDim.x, n = a.n;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = nb * blockDim.x;
    double *r = a.scratch, *z = r + kMaxRows, *p = z + kMaxRows, *Ap = p + kMaxRows, *dinv = Ap + kMaxRows;
    double *partA = dinv + kMaxRows, *partB = partA + kMaxBlocks, *partC = partB + kMaxBlocks,
           *partD = partC + kMaxBlocks;
    double *out = partD + kMaxBlocks;
    double ra, rb;
    // D^-1, r = b - A x, z = D^-1 r, p = z (every scratch value written before it is read)
    double rz = 0.0, rr = 0.0, bb = 0.0;
    for (int i = gtid; i < n; i += gstride) {
        double s = 0.0, d = 0.0;
        for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k) {
            const int j = a.col[k];
            s = fma(a.val[k], a.x[j], s);
            if (j == i) d = a.val[k];
        }
        const double di = d != 0.0 ? 1.0 / d : 1.0;
        const double bi = a.b[i], ri = bi - s, zi = di * ri;
        dinv[i] = di; r[i] = ri; z[i] = zi; p[i] = zi;
        rz = fma(ri, zi, rz); rr = fma(ri, ri, rr); bb = fma(bi, bi, bb);
    }
    na_block_sum2(rz, rr, sh, ra, rb);
    if (threadIdx.x == 0) { partA[blockIdx.x] = ra; partB[blockIdx.x] = rb; }
    na_block_sum2(bb, 0.0, sh, ra, rb);
    if (threadIdx.x == 0) { partC[blockIdx.x] = ra; partD[blockIdx.x] = 0.0; }
    grid.sync();
    double t_rz = 0.0, t_rr = 0.0, t_bb = 0.0, t_tol2 = 0.0;
    int t_it = 0, t_status = 1;
    na_grid_sum2(partA, partB, nb, sh, ra, rb);
    if (threadIdx.x == 0) { t_rz = ra; t_rr = rb; }
    na_grid_sum2(partC, partD, nb, sh, ra, rb);
    if (threadIdx.x == 0) {
        t_bb = ra;
        const double tol = fmax(a.rtol * sqrt(t_bb), a.atol);
        t_tol2 = tol * tol;
        if (t_rr <= t_tol2) t_status = 0;
        scal[1] = (t_status == 1 && a.max_iter > 0) ? 1.0 : 0.0;
    }
    __syncthreads();
    grid.sync();
    while (scal[1] != 0.0) {
        double pap = 0.0;
        for (int i = gtid; i < n; i += gstride) {
            double s = 0.0;
            for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k) s = fma(a.val[k], __ldcg(p + a.col[k]), s);
            Ap[i] = s;
            pap = fma(__ldcg(p + i), s, pap);
        }
        na_block_sum2(pap, 0.0, sh, ra, rb);
        if (threadIdx.x == 0) { partA[blockIdx.x] = ra; partD[blockIdx.x] = 0.0; }
        grid.sync();
        na_grid_sum2(partA, partD, nb, sh, ra, rb);
        if (threadIdx.x == 0) {
            ++t_it;
            if (!(ra > 0.0)) { t_status = 2; scal[1] = 0.0; }
            else scal[0] = t_rz / ra;
        }
        __syncthreads();
        if (scal[1] == 0.0) break;
        const double alpha = scal[0];
        double rzn = 0.0, rrn = 0.0;
        for (int i = gtid; i < n; i += gstride) {
            a.x[i] = fma(alpha, __ldcg(p + i), a.x[i]);
            const double ri = fma(-alpha, Ap[i], r[i]);
            const double zi = dinv[i] * ri;
            r[i] = ri; z[i] = zi;
            rzn = fma(ri, zi, rzn); rrn = fma(ri, ri, rrn);
        }
        na_block_sum2(rzn, rrn, sh, ra, rb);
        if (threadIdx.x == 0) { partB[blockIdx.x] = ra; partC[blockIdx.x] = rb; }
        grid.sync();
        na_grid_sum2(partB, partC, nb, sh, ra, rb);
        if (threadIdx.x == 0) {
            t_rr = rb;
            if (t_rr <= t_tol2) { t_status = 0; scal[1] = 0.0; }
            else if (t_it >= a.max_iter) { t_status = 1; scal[1] = 0.0; }
            scal[0] = ra / t_rz;
            t_rz = ra;
        }
        __syncthreads();
        if (scal[1] == 0.0) break;
        const double beta = scal[0];
        for (int i = gtid; i < n; i += gstride) p[i] = fma(beta, __ldcg(p + i), z[i]);
        grid.sync();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        out[0] = (double)t_it;
        out[1] = (double)t_status;
        out[2] = t_rr;
        out[3] = t_bb;
    }
}

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double *g_scratch_ptr[kMaxDevices] = {};
int g_grid_blocks[kMaxDevices] = {};

}  // namespace

}  // namespace pg

extern "C" int pg_pcg_solve_noalloc(int32_t n, const int32_t *rowptr, const int32_t *col, const double *val,
                                    const double *b, double *x, double rtol, double atol, int32_t max_iter,
                                    void *stream, int32_t *iterations, double *residual) {
    using namespace pg;
    if (n <= 0 || !rowptr || !col || !val || !b || !x)
        return fail(PG_ERR_ARG, "pg_pcg_solve_noalloc: empty system or NULL pointer");
    if (n > kMaxRows)
        return fail(PG_ERR_ARG, "pg_pcg_solve_noalloc: " + std::to_string(n) + " rows exceed the static scratch limit of " +
                                    std::to_string(kMaxRows) + " rows");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(PG_ERR_CUDA, std::string("pg_pcg_solve_noalloc: no usable current device: ") + cudaGetErrorString(e));
    {
        // once per device, with that device current
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_ptr[dev]) {
            void *ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr)
                return fail(PG_ERR_CUDA, std::string("pg_pcg_solve_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            int per_sm = 0, sms = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_csr_noalloc, kNaThreads, 0);
            if (e != cudaSuccess) return fail(PG_ERR_CUDA, std::string("pg_pcg_solve_noalloc: ") + cudaGetErrorString(e));
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return fail(PG_ERR_CUDA, std::string("pg_pcg_solve_noalloc: ") + cudaGetErrorString(e));
            int g = std::max(1, std::min(per_sm, 2)) * std::max(1, sms);
            g_grid_blocks[dev] = std::min(g, kMaxBlocks);
            g_scratch_ptr[dev] = static_cast<double *>(ptr);
        }
    }
    double *scratch = g_scratch_ptr[dev];
    int nb = g_grid_blocks[dev];
    const int need = (n + kNaThreads - 1) / kNaThreads;
    if (need < nb) nb = need;
    NoAllocArgs a{n, rowptr, col, val, b, x, rtol, atol, max_iter, scratch};
    void *params[] = {&a};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    count_launches(1);
    e = cudaLaunchCooperativeKernel((const void *)k_pcg_csr_noalloc, dim3(nb), dim3(kNaThreads), params, 0, st);
    if (e != cudaSuccess)
        return fail(PG_ERR_CUDA, std::string("pg_pcg_solve_noalloc: launch: ") + cudaGetErrorString(e));
    double out[4] = {0, 0, 0, 0};
    e = cudaMemcpyAsync(out, scratch + 5 * (size_t)kMaxRows + 4 * (size_t)kMaxBlocks, sizeof(out),
                        cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(PG_ERR_CUDA, std::string("pg_pcg_solve_noalloc: ") + cudaGetErrorString(e));
    if (iterations) *iterations = (int32_t)out[0];
    if (residual) *residual = std::sqrt(out[2]);
    const int status = (int)out[1];
    if (status == 1) return fail(PG_ERR_NOT_CONVERGED, "pg_pcg_solve_noalloc: iteration cap reached");
    if (status == 2) return fail(PG_ERR_NOT_CONVERGED, "pg_pcg_solve_noalloc: breakdown (p.Ap <= 0)");
    return PG_OK;
}
