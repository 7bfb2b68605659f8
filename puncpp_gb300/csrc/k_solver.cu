// Field kernels: DG0 electric field, Poisson right-hand side, a persistent
// cooperative Jacobi-preconditioned CG, and object image charges.
// Built with --fmad=false so E matches a CPU evaluation bit for bit.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "pg_device.cuh"
#include "pg_reduce.cuh"

namespace cg = cooperative_groups;

namespace pg {

namespace {

constexpr int kThreads = 256;


// E = -grad(phi) on each cell (EFieldDG0::solve, punc/src/efield.cpp:95-99):
// grad(phi) = (phi0-phi3) g0 + (phi1-phi3) g1 + (phi2-phi3) g2 with g_k the
// gradient rows of the barycentric matrix (g3 = -(g0+g1+g2)); E0 added after.
__global__ void k_efield(DevMesh m, const double *__restrict__ phi, double e0x, double e0y, double e0z) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.nc) return;
    double ex, ey, ez;
    dg0_field_f64(m.bary + 12 * (size_t)c, m.dofs[c], phi, e0x, e0y, e0z, ex, ey, ez);
    double2 *E = reinterpret_cast<double2 *>(m.E) + 2 * (size_t)c;
    E[0] = make_double2(ex, ey);
    E[1] = make_double2(ez, 0.0);
    if (m.E_f) reinterpret_cast<float4 *>(m.E_f)[c] = make_float4((float)ex, (float)ey, (float)ez, 0.0f);
}

// b = M rho on free rows, minus the Dirichlet columns moved to the right-hand
// side; b = g on Dirichlet rows (PoissonSolver::solve, punc/src/poisson.cpp:343-362,
// with the BC rows eliminated symmetrically).  M in SELL-32 (one thread per
// row, the row's entries in their CSR order; padding: value 0, own column).
__global__ void k_rhs(int32_t n, const int64_t *__restrict__ sptr, const int32_t *__restrict__ swidth,
                      const int32_t *__restrict__ scol, const double *__restrict__ sval,
                      const double *__restrict__ rho, const int32_t *__restrict__ bc_kind,
                      const double *__restrict__ bc_value, const double *__restrict__ w_ext,
                      const double *__restrict__ w_obj, const double *__restrict__ obj_pot, int32_t n_obj,
                      int32_t use_ext, double *__restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = bc_kind[i];
    if (k == 0) { b[i] = use_ext ? bc_value[i] : 0.0; return; }
    if (k > 0) { b[i] = obj_pot[k - 1]; return; }
    const int64_t base = __ldg(sptr + (i >> 5)) + (i & 31);
    const int w = __ldg(swidth + (i >> 5));
    double s = 0.0;
    for (int e = 0; e < w; ++e) s += __ldg(sval + base + 32 * e) * __ldg(rho + __ldg(scol + base + 32 * e));
    if (use_ext) s = s - w_ext[i];
    for (int o = 0; o < n_obj; ++o) s = s - obj_pot[o] * w_obj[(size_t)o * n + i];
    b[i] = s;
}

__global__ void k_set_bc(const int32_t *__restrict__ bc_kind, const double *__restrict__ bc_value,
                         const double *__restrict__ obj_pot, int32_t n, double *__restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = bc_kind[i];
    if (k == 0) x[i] = bc_value ? bc_value[i] : 0.0;
    else if (k > 0) x[i] = obj_pot[k - 1];
}

// Sum of one value per block, then every block reads all block partials in
// the same order, so all blocks hold the same total.
__device__ double block_reduce(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (wid == 0) {
        s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) sh[0] = s;
    }
    __syncthreads();
    s = sh[0];
    __syncthreads();
    return s;
}

// Preconditioned CG with the Jacobi preconditioner, all iterations in one
// cooperative launch.  Per iteration (three grid-wide barriers):
//   A: Ap = A p (SELL-32 rows, one FMA and one gather per entry), partial p.Ap
//   B: x += alpha p, r -= alpha Ap, z = D^-1 r, partials r.z and r.r
//   C: p = z + beta p
// Stops when ||r||^2 <= max(rtol ||b||, atol)^2 (unpreconditioned residual).
// The solver is checked against a direct solve to a tolerance, so it uses
// FMAs (GB300's FP64 rate makes FP64 instruction count the bound here).
__global__ void __launch_bounds__(kPcgThreads, 2) k_pcg(PcgArgs a) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[2 * kPcgThreads + 16];
    __shared__ double scal[4];      // alpha or beta, status, ...
    const int nb = gridDim.x;
    const int n = a.n;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gstride = nb * blockDim.x;
    double *partA = a.partials;
    double *partB = a.partials + nb;
    double *partC = a.partials + 2 * nb;
    double *partD = a.partials + 3 * nb;
    double *p = a.p0;
    double ra, rb;

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
    // r = b - A x, z = D^-1 r, p = z
    double rz = 0.0, rr = 0.0, bb = 0.0;
    for (int i = gtid; i < n; i += gstride) {
        double s = 0.0;
        const int64_t base = a.slice_ptr[i >> 5] + (i & 31);
        const int w = a.slice_width[i >> 5];
        for (int k = 0; k < w; ++k) s = fma(__ldg(a.val + base + 32 * k), a.x[__ldg(a.col + base + 32 * k)], s);
        const double bi = a.b[i];
        const double ri = bi - s;
        const double zi = a.dinv[i] * ri;
        a.r[i] = ri; a.z[i] = zi; p[i] = zi;
        rz = fma(ri, zi, rz); rr = fma(ri, ri, rr); bb = fma(bi, bi, bb);
    }
    block_sum2(rz, rr, sh, ra, rb);
    if (threadIdx.x == 0) { partA[blockIdx.x] = ra; partB[blockIdx.x] = rb; }
    block_sum2(bb, 0.0, sh, ra, rb);
    if (threadIdx.x == 0) partC[blockIdx.x] = ra;
    grid.sync();
    // thread 0 keeps the scalars: rz, tol^2, iteration, status
    double t_rz = 0.0, t_tol2 = 0.0, t_rr = 0.0, t_bb = 0.0;
    int t_it = 0, t_status = 1;
    grid_sum2(partA, partB, nb, sh, ra, rb);
    if (threadIdx.x == 0) { t_rz = ra; t_rr = rb; }
    grid_sum2(partC, nullptr, nb, sh, ra, rb);
    if (threadIdx.x == 0) {
        t_bb = ra;
        const double tol = fmax(a.rtol * sqrt(t_bb), a.atol);
        t_tol2 = tol * tol;
        if (t_rr <= t_tol2) t_status = 0;
        if (a.max_iter <= 0 && t_status == 1) t_status = 1;
        scal[1] = (t_status == 1 && a.max_iter > 0) ? 1.0 : 0.0;
    }
    __syncthreads();
    grid.sync();
    while (scal[1] != 0.0) {
        // A
        double pap = 0.0;
        for (int i = gtid; i < n; i += gstride) {
            double s = 0.0;
            const int64_t base = a.slice_ptr[i >> 5] + (i & 31);
            const int w = a.slice_width[i >> 5];
#pragma unroll 4
            for (int k = 0; k < w; ++k)
                s = fma(__ldg(a.val + base + 32 * k), __ldcg(p + __ldg(a.col + base + 32 * k)), s);
            a.Ap[i] = s;
            pap = fma(__ldcg(p + i), s, pap);
        }
        block_sum2(pap, 0.0, sh, ra, rb);
        if (threadIdx.x == 0) partA[blockIdx.x] = ra;
        grid.sync();
        grid_sum2(partA, nullptr, nb, sh, ra, rb);
        if (threadIdx.x == 0) {
            ++t_it;
            if (!(ra > 0.0)) { t_status = 2; scal[1] = 0.0; scal[0] = 0.0; }
            else scal[0] = t_rz / ra;
        }
        __syncthreads();
        if (scal[1] == 0.0) break;
        const double alpha = scal[0];
        // B
        double rzn = 0.0, rrn = 0.0;
        for (int i = gtid; i < n; i += gstride) {
            const double pi = __ldcg(p + i);
            a.x[i] = fma(alpha, pi, a.x[i]);
            const double ri = fma(-alpha, a.Ap[i], a.r[i]);
            const double zi = a.dinv[i] * ri;
            a.r[i] = ri; a.z[i] = zi;
            rzn = fma(ri, zi, rzn); rrn = fma(ri, ri, rrn);
        }
        block_sum2(rzn, rrn, sh, ra, rb);
        if (threadIdx.x == 0) { partB[blockIdx.x] = ra; partC[blockIdx.x] = rb; }
        grid.sync();
        grid_sum2(partB, partC, nb, sh, ra, rb);
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
        // C
        for (int i = gtid; i < n; i += gstride) p[i] = fma(beta, __ldcg(p + i), a.z[i]);
        grid.sync();
    }
    if (a.remove_mean) {
        grid.sync();
        double s = 0.0;
        for (int i = gtid; i < n; i += gstride) s += a.x[i];
        block_sum2(s, 0.0, sh, ra, rb);
        if (threadIdx.x == 0) partD[blockIdx.x] = ra;
        grid.sync();
        grid_sum2(partD, nullptr, nb, sh, ra, rb);
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
    }
}

// Mixed-precision PCG with reliable updates: the Krylov recurrence (SpMV,
// residual, preconditioned residual, search direction) in FP32, the solution
// accumulated in FP64, every inner product reduced in FP64, and the residual
// replaced by the FP64 true residual b - A x whenever the recursive one has
// dropped tenfold since the last replacement.  It stops only when the FP64
// true residual meets ||r|| <= max(rtol ||b||, atol).
__global__ void __launch_bounds__(kPcgThreads, 2) k_pcg_rel(PcgArgs a) {
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
    double t_rz = 0.0, t_tol2 = 0.0, t_rr = 0.0, t_bb = 0.0, t_rmax = 0.0;
    int t_it = 0, t_status = 1, t_updates = 0;
    // true residual in FP64, copied to the FP32 recurrence; p = z on the first pass
    for (int pass = 0;; ++pass) {
        double rz = 0.0, rr = 0.0, bb = 0.0;
        for (int i = gtid; i < n; i += gstride) {
            double s = 0.0;
            const int64_t base = a.slice_ptr[i >> 5] + (i & 31);
            const int w = a.slice_width[i >> 5];
            // x is updated by other blocks between passes: read it through L2
#pragma unroll 4
            for (int k = 0; k < w; ++k) s = fma(__ldg(a.val + base + 32 * k), __ldcg(a.x + __ldg(a.col + base + 32 * k)), s);
            const double bi = a.b[i];
            const double ri = bi - s;
            const float r32 = (float)ri;
            const float z32 = a.dinv32[i] * r32;
            a.r32[i] = r32; a.z32[i] = z32;
            if (pass == 0) a.p32[i] = z32;
            rz = fma((double)r32, (double)z32, rz); rr = fma(ri, ri, rr);
            if (pass == 0) bb = fma(bi, bi, bb);
        }
        block_sum2(rz, rr, sh, ra, rb);
        if (threadIdx.x == 0) { partA[blockIdx.x] = ra; partB[blockIdx.x] = rb; }
        if (pass == 0) {
            block_sum2(bb, 0.0, sh, ra, rb);
            if (threadIdx.x == 0) partC[blockIdx.x] = ra;
        }
        grid.sync();
        grid_sum2(partA, partB, nb, sh, ra, rb);
        if (threadIdx.x == 0) {
            const double rz_new = ra;
            // the recurrence's ||r|| fell tenfold since the last replacement
            // but the true one by less than half that: the FP32 recurrence's
            // attainable accuracy (status 3, as k_pcg_amg)
            scal[2] = (pass > 0 && rb > 0.25 * t_rr) ? 1.0 : 0.0;
            t_rr = rb;
            if (pass > 0) ++t_updates;
            // keep the search direction; its coefficient uses the replaced r.z
            scal[0] = pass > 0 ? rz_new / t_rz : 0.0;
            t_rz = rz_new;
            t_rmax = t_rr;
        }
        if (pass == 0) {
            grid_sum2(partC, nullptr, nb, sh, ra, rb);
            if (threadIdx.x == 0) {
                t_bb = ra;
                const double tol = fmax(a.rtol * sqrt(t_bb), a.atol);
                t_tol2 = tol * tol;
            }
        }
        if (threadIdx.x == 0) {
            if (t_rr <= t_tol2) { t_status = 0; scal[1] = 0.0; }
            else if (t_it >= a.max_iter) { t_status = 1; scal[1] = 0.0; }
            else if (scal[2] != 0.0) { t_status = 3; scal[1] = 0.0; }
            else scal[1] = 1.0;
        }
        __syncthreads();
        if (scal[1] == 0.0) break;
        if (pass > 0) {
            // p = z + beta p with the replaced residual
            const float beta = (float)scal[0];
            for (int i = gtid; i < n; i += gstride) a.p32[i] = fmaf(beta, __ldcg(a.p32 + i), a.z32[i]);
        }
        grid.sync();
        // FP32 recurrence until the residual has dropped tenfold (or converged)
        bool replace = false;
        while (!replace) {
            float pap32 = 0.0f;
            for (int i = gtid; i < n; i += gstride) {
                float s = 0.0f;
                const int64_t base = a.slice_ptr[i >> 5] + (i & 31);
                const int w = a.slice_width[i >> 5];
#pragma unroll 4
                for (int k = 0; k < w; ++k)
                    s = fmaf(__ldg(a.val32 + base + 32 * k), __ldcg(a.p32 + __ldg(a.col + base + 32 * k)), s);
                a.Ap32[i] = s;
                pap32 = fmaf(__ldcg(a.p32 + i), s, pap32);
            }
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
            const double alpha = scal[0];
            const float alpha32 = (float)alpha;
            float rz32 = 0.0f, rr32 = 0.0f;
            for (int i = gtid; i < n; i += gstride) {
                const float pi = __ldcg(a.p32 + i);
                a.x[i] = fma(alpha, (double)pi, a.x[i]);
                const float ri = fmaf(-alpha32, a.Ap32[i], a.r32[i]);
                const float zi = a.dinv32[i] * ri;
                a.r32[i] = ri; a.z32[i] = zi;
                rz32 = fmaf(ri, zi, rz32); rr32 = fmaf(ri, ri, rr32);
            }
            block_sum2((double)rz32, (double)rr32, sh, ra, rb);
            if (threadIdx.x == 0) { partB[blockIdx.x] = ra; partC[blockIdx.x] = rb; }
            grid.sync();
            grid_sum2(partB, partC, nb, sh, ra, rb);
            if (threadIdx.x == 0) {
                const double rr_rec = rb;
                // replace the residual after a tenfold drop, at the tolerance, or at the cap;
                // on a replacement r.z of the previous step stays for the next beta
                const bool rep = rr_rec <= 0.01 * t_rmax || rr_rec <= t_tol2 || t_it >= a.max_iter;
                scal[2] = rep ? 1.0 : 0.0;
                if (!rep) { scal[0] = ra / t_rz; t_rz = ra; }
            }
            __syncthreads();
            replace = scal[2] != 0.0;
            if (replace) break;
            const float beta = (float)scal[0];
            for (int i = gtid; i < n; i += gstride) a.p32[i] = fmaf(beta, __ldcg(a.p32 + i), a.z32[i]);
            grid.sync();
        }
        if (scal[1] == 0.0) break;      // breakdown
        grid.sync();
    }
    if (a.remove_mean) {
        grid.sync();
        double s = 0.0;
        for (int i = gtid; i < n; i += gstride) s += a.x[i];
        block_sum2(s, 0.0, sh, ra, rb);
        if (threadIdx.x == 0) partD[blockIdx.x] = ra;
        grid.sync();
        grid_sum2(partD, nullptr, nb, sh, ra, rb);
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

// Image charge of each object: sum over its facets of
// eps0 * area * grad(phi_T) . n (the Charge.ufl ds-integral for P1,
// CircuitCM::post_solve, punc/src/object_CM.cpp:328-337).  One block, facets
// in list order, per-object partial sums combined in a fixed tree order.
__global__ void k_image_charge(DevMesh m, const double *__restrict__ phi, const double *__restrict__ of, int32_t nf,
                               int32_t n_obj, double eps0, double *__restrict__ out) {
    __shared__ double sh[32];
    for (int o = 0; o < n_obj; ++o) {
        double v = 0.0;
        for (int f = threadIdx.x; f < nf; f += blockDim.x) {
            const double *r = of + 7 * (size_t)f;
            if ((int)r[1] != o) continue;
            const int c = (int)r[0];
            const int4 d = m.dofs[c];
            const double p3 = phi[d.w];
            const double a = phi[d.x] - p3, b = phi[d.y] - p3, e = phi[d.z] - p3;
            const double *A = m.bary + 12 * (size_t)c;
            const double gx = a * A[1] + b * A[5] + e * A[9];
            const double gy = a * A[2] + b * A[6] + e * A[10];
            const double gz = a * A[3] + b * A[7] + e * A[11];
            const double gn = gx * r[3] + gy * r[4] + gz * r[5];
            v += (eps0 * r[2]) * gn;
        }
        v = block_reduce(v, sh);
        if (threadIdx.x == 0) out[o] = v;
    }
}

// phi = phi0 + sum_k V_k L_k: the solution with object potentials V from the
// one with zero potentials and the unit-potential Laplace solutions L_k.
__global__ void k_superpose(const double *__restrict__ phi0, const double *__restrict__ lap, Pots pots,
                            const int32_t *__restrict__ rng, int32_t n, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = phi0[i];
    for (int k = 0; k < pots.n; ++k)
        if (!rng || (i >= rng[2 * k] && i < rng[2 * k + 1])) v = v + pots.v[k] * lap[(size_t)k * n + i];
    out[i] = v;
}

}  // namespace

void launch_superpose(const double *phi0, const double *lap, const Pots &pots, const int32_t *rng, int32_t n,
                      double *out, cudaStream_t st) {
    count_launches(1);
    k_superpose<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(phi0, lap, pots, rng, n, out);
}

void launch_efield(const DevMesh &m, const double *phi, const double E0[3], cudaStream_t st) {
    if (m.nc <= 0) return;
    count_launches(1);
    k_efield<<<(m.nc + kThreads - 1) / kThreads, kThreads, 0, st>>>(m, phi, E0[0], E0[1], E0[2]);
}

void launch_rhs(const DevMesh &m, const int64_t *msptr, const int32_t *mswidth, const int32_t *mscol,
                const double *msval, const double *rho, const int32_t *bc_kind, const double *bc_value,
                const double *w_ext, const double *w_obj, const double *obj_pot, int32_t n_obj, int32_t use_ext,
                double *b, cudaStream_t st) {
    count_launches(1);
    k_rhs<<<(m.ndof + kThreads - 1) / kThreads, kThreads, 0, st>>>(m.ndof, msptr, mswidth, mscol, msval, rho, bc_kind,
                                                                    bc_value, w_ext, w_obj, obj_pot, n_obj, use_ext, b);
}

void launch_set_bc(const int32_t *bc_kind, const double *bc_value, const double *obj_pot, int32_t n, double *x,
                   cudaStream_t st) {
    count_launches(1);
    k_set_bc<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(bc_kind, bc_value, obj_pot, n, x);
}

int pcg_grid_blocks() {
    static int g = 0;
    if (g == 0) {
        int per_sm = 0, per_sm_rel = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, kPcgThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_rel, k_pcg_rel, kPcgThreads, 0);
        if (per_sm_rel < per_sm) per_sm = per_sm_rel;
        if (per_sm < 1) per_sm = 1;
        if (per_sm > 4) per_sm = 4;
        g = per_sm * sm_count();
    }
    return g;
}

int launch_pcg(const PcgArgs &a, cudaStream_t st) {
    int nb = pcg_grid_blocks();
    const int need = (a.n + kPcgThreads - 1) / kPcgThreads;
    if (need < nb) nb = need < 1 ? 1 : need;
    PcgArgs arg = a;
    void *params[] = {&arg};
    count_launches(1);
    const void *fn = a.val32 ? (const void *)k_pcg_rel : (const void *)k_pcg;
    cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(nb), dim3(kPcgThreads), params, 0, st);
    return e == cudaSuccess ? 0 : (int)e;
}

void launch_image_charge(const DevMesh &m, const double *phi, const double *ofacets, int32_t n_ofacets, int32_t n_obj,
                         double eps0, double *out, cudaStream_t st) {
    if (n_obj <= 0) return;
    count_launches(1);
    k_image_charge<<<1, 1024, 0, st>>>(m, phi, ofacets, n_ofacets, n_obj, eps0, out);
}

}  // namespace pg
