// FP64 reductions of the persistent PCG kernels (block size kPcgThreads).
#pragma once

#include "pg_device.cuh"

namespace pg {

constexpr int kPcgThreads = 512;

// ---- PCG reductions ---------------------------------------------------------
// GB300 executes a warp-wide FP64 add in ~64 cycles of one SM sub-partition,
// so the reductions keep FP64 work off most warps: the 512 per-thread partials
// go to shared memory, warps 0-3 (one per sub-partition) each sum a quarter,
// and thread 0 alone forms the scalars of the iteration.

// Sum of two per-thread values over the block; valid in thread 0.
__device__ __forceinline__ void block_sum2(double a, double b, double *sh, double &ra, double &rb) {
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    sh[t] = a;
    sh[kPcgThreads + t] = b;
    __syncthreads();
    if (w < 4) {
        const int q = kPcgThreads / 4;
        double sa = 0.0, sb = 0.0;
        for (int k = lane; k < q; k += 32) { sa += sh[w * q + k]; sb += sh[kPcgThreads + w * q + k]; }
        for (int o = 16; o > 0; o >>= 1) {
            sa += __shfl_down_sync(0xffffffffu, sa, o);
            sb += __shfl_down_sync(0xffffffffu, sb, o);
        }
        if (lane == 0) { sh[2 * kPcgThreads + w] = sa; sh[2 * kPcgThreads + 4 + w] = sb; }
    }
    __syncthreads();
    if (t == 0) {
        const double *r = sh + 2 * kPcgThreads;
        ra = (r[0] + r[1]) + (r[2] + r[3]);
        rb = (r[4] + r[5]) + (r[6] + r[7]);
    }
}

// Sum of the per-block partials of two quantities (all blocks read the same
// partials in the same order, so every block gets the same totals); valid in thread 0.
__device__ __forceinline__ void grid_sum2(const double *pa, const double *pb, int nb, double *sh, double &ra, double &rb) {
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    if (w < 4) {
        double sa = 0.0, sb = 0.0;
        for (int k = w * 32 + lane; k < nb; k += 128) { sa += __ldcg(pa + k); if (pb) sb += __ldcg(pb + k); }
        for (int o = 16; o > 0; o >>= 1) {
            sa += __shfl_down_sync(0xffffffffu, sa, o);
            sb += __shfl_down_sync(0xffffffffu, sb, o);
        }
        if (lane == 0) { sh[2 * kPcgThreads + 8 + w] = sa; sh[2 * kPcgThreads + 12 + w] = sb; }
    }
    __syncthreads();
    if (t == 0) {
        const double *r = sh + 2 * kPcgThreads + 8;
        ra = (r[0] + r[1]) + (r[2] + r[3]);
        rb = (r[4] + r[5]) + (r[6] + r[7]);
    }
}

}  // namespace pg
