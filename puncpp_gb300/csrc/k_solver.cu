// Field kernels: DG0 electric field, Poisson right-hand side, a persistent
// cooperative Jacobi-preconditioned CG, and object image charges.
// Built with --fmad=false so E matches a CPU evaluation bit for bit.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "pg_device.cuh"

namespace cg = cooperative_groups;

namespace pg {

namespace {

constexpr int kThreads = 256;
constexpr int kPcgThreads = 512;

// E = -grad(phi) on each cell (EFieldDG0::solve, punc/src/efield.cpp:95-99):
// grad(phi) = (phi0-phi3) g0 + (phi1-phi3) g1 + (phi2-phi3) g2 with g_k the
// gradient rows of the barycentric matrix (g3 = -(g0+g1+g2)); E0 added after.
__global__ void k_efield(DevMesh m, const double *__restrict__ phi, double e0x, double e0y, double e0z) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.nc) return;
    const int4 d = m.dofs[c];
    const double p3 = phi[d.w];
    const double a = phi[d.x] - p3, b = phi[d.y] - p3, e = phi[d.z] - p3;
    const double *A = m.bary + 12 * (size_t)c;
    const double gx = a * A[1] + b * A[5] + e * A[9];
    const double gy = a * A[2] + b * A[6] + e * A[10];
    const double gz = a * A[3] + b * A[7] + e * A[11];
    double2 *E = reinterpret_cast<double2 *>(m.E) + 2 * (size_t)c;
    E[0] = make_double2(-gx + e0x, -gy + e0y);
    E[1] = make_double2(-gz + e0z, 0.0);
}

// b = M rho on free rows, minus the Dirichlet columns moved to the right-hand
// side; b = g on Dirichlet rows (PoissonSolver::solve, punc/src/poisson.cpp:343-362,
// with the BC rows eliminated symmetrically).
__global__ void k_rhs(int32_t n, const int32_t *__restrict__ mrow, const int32_t *__restrict__ mcol,
                      const double *__restrict__ mval, const double *__restrict__ rho,
                      const int32_t *__restrict__ bc_kind, const double *__restrict__ bc_value,
                      const double *__restrict__ w_ext, const double *__restrict__ w_obj,
                      const double *__restrict__ obj_pot, int32_t n_obj, int32_t use_ext, double *__restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = bc_kind[i];
    if (k == 0) { b[i] = use_ext ? bc_value[i] : 0.0; return; }
    if (k > 0) { b[i] = obj_pot[k - 1]; return; }
    double s = 0.0;
    for (int j = mrow[i]; j < mrow[i + 1]; ++j) s += mval[j] * rho[mcol[j]];
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

__device__ double grid_total(const double *part, int nb, double *sh) {
    double v = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) v += __ldcg(part + i);
    return block_reduce(v, sh);
}

// Preconditioned CG with the Jacobi preconditioner, all iterations in one
// cooperative launch.  Per iteration:
//   phase A: p_new = z + beta p_old (on the fly in the gather), Ap = A p_new,
//            partial p_new.Ap
//   phase B: x += alpha p_new, r -= alpha Ap, z = D^-1 r, partials r.z, r.r
// Stops when ||r|| <= max(rtol ||b||, atol) (unpreconditioned residual).
__global__ void __launch_bounds__(kPcgThreads) k_pcg(PcgArgs a) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double sh[32];
    const int nb = gridDim.x;
    const int n = a.n;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gstride = nb * blockDim.x;
    double *partA = a.partials;
    double *partB = a.partials + nb;
    double *partC = a.partials + 2 * nb;
    double *partD = a.partials + 3 * nb;

    if (a.remove_mean) {
        double s = 0.0;
        for (int i = gtid; i < n; i += gstride) s += a.b[i];
        s = block_reduce(s, sh);
        if (threadIdx.x == 0) partD[blockIdx.x] = s;
        grid.sync();
        const double mean = grid_total(partD, nb, sh) / (double)n;
        for (int i = gtid; i < n; i += gstride) a.b[i] = a.b[i] - mean;
        grid.sync();
    }
    // r = b - A x, z = D^-1 r, p_old = 0.
    double rz = 0.0, rr = 0.0, bb = 0.0;
    for (int i = gtid; i < n; i += gstride) {
        double s = 0.0;
        for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k) s += a.val[k] * a.x[a.col[k]];
        const double bi = a.b[i];
        const double ri = bi - s;
        const double zi = a.dinv[i] * ri;
        a.r[i] = ri; a.z[i] = zi; a.p0[i] = 0.0;
        rz += ri * zi; rr += ri * ri; bb += bi * bi;
    }
    rz = block_reduce(rz, sh);
    rr = block_reduce(rr, sh);
    bb = block_reduce(bb, sh);
    if (threadIdx.x == 0) { partA[blockIdx.x] = rz; partB[blockIdx.x] = rr; partC[blockIdx.x] = bb; }
    grid.sync();
    rz = grid_total(partA, nb, sh);
    rr = grid_total(partB, nb, sh);
    bb = grid_total(partC, nb, sh);
    const double tol = fmax(a.rtol * sqrt(bb), a.atol);
    int status = 1, it = 0;
    double beta = 0.0;
    double *pold = a.p0, *pnew = a.p1;
    if (sqrt(rr) <= tol) status = 0;
    grid.sync();
    while (status == 1 && it < a.max_iter) {
        ++it;
        // phase A
        double pap = 0.0;
        for (int i = gtid; i < n; i += gstride) {
            double s = 0.0;
            for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k) {
                const int j = a.col[k];
                const double pj = __ldcg(a.z + j) + beta * __ldcg(pold + j);
                s += a.val[k] * pj;
            }
            const double pi = __ldcg(a.z + i) + beta * __ldcg(pold + i);
            pnew[i] = pi;
            a.Ap[i] = s;
            pap += pi * s;
        }
        pap = block_reduce(pap, sh);
        if (threadIdx.x == 0) partA[blockIdx.x] = pap;
        grid.sync();
        pap = grid_total(partA, nb, sh);
        if (!(pap > 0.0)) { status = 2; break; }
        const double alpha = rz / pap;
        // phase B
        double rzn = 0.0, rrn = 0.0;
        for (int i = gtid; i < n; i += gstride) {
            const double pi = pnew[i];
            const double api = a.Ap[i];
            a.x[i] = a.x[i] + alpha * pi;
            const double ri = a.r[i] - alpha * api;
            const double zi = a.dinv[i] * ri;
            a.r[i] = ri; a.z[i] = zi;
            rzn += ri * zi; rrn += ri * ri;
        }
        rzn = block_reduce(rzn, sh);
        rrn = block_reduce(rrn, sh);
        if (threadIdx.x == 0) { partB[blockIdx.x] = rzn; partC[blockIdx.x] = rrn; }
        grid.sync();
        rzn = grid_total(partB, nb, sh);
        rr = grid_total(partC, nb, sh);
        if (sqrt(rr) <= tol) { status = 0; break; }
        beta = rzn / rz;
        rz = rzn;
        double *t = pold; pold = pnew; pnew = t;
        grid.sync();
    }
    if (a.remove_mean) {
        grid.sync();
        double s = 0.0;
        for (int i = gtid; i < n; i += gstride) s += a.x[i];
        s = block_reduce(s, sh);
        if (threadIdx.x == 0) partD[blockIdx.x] = s;
        grid.sync();
        const double mean = grid_total(partD, nb, sh) / (double)n;
        for (int i = gtid; i < n; i += gstride) a.x[i] = a.x[i] - mean;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *a.out_iter = it;
        *a.out_status = status;
        *a.out_rr = rr;
        *a.out_bb = bb;
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

}  // namespace

void launch_efield(const DevMesh &m, const double *phi, const double E0[3], cudaStream_t st) {
    if (m.nc <= 0) return;
    count_launches(1);
    k_efield<<<(m.nc + kThreads - 1) / kThreads, kThreads, 0, st>>>(m, phi, E0[0], E0[1], E0[2]);
}

void launch_rhs(const DevMesh &m, const int32_t *mrow, const int32_t *mcol, const double *mval, const double *rho,
                const int32_t *bc_kind, const double *bc_value, const double *w_ext, const double *w_obj,
                const double *obj_pot, int32_t n_obj, int32_t use_ext, double *b, cudaStream_t st) {
    count_launches(1);
    k_rhs<<<(m.ndof + kThreads - 1) / kThreads, kThreads, 0, st>>>(m.ndof, mrow, mcol, mval, rho, bc_kind, bc_value,
                                                                    w_ext, w_obj, obj_pot, n_obj, use_ext, b);
}

void launch_set_bc(const int32_t *bc_kind, const double *bc_value, const double *obj_pot, int32_t n, double *x,
                   cudaStream_t st) {
    count_launches(1);
    k_set_bc<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(bc_kind, bc_value, obj_pot, n, x);
}

int pcg_grid_blocks() {
    static int g = 0;
    if (g == 0) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, kPcgThreads, 0);
        if (per_sm < 1) per_sm = 1;
        if (per_sm > 2) per_sm = 2;
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
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_pcg, dim3(nb), dim3(kPcgThreads), params, 0, st);
    return e == cudaSuccess ? 0 : (int)e;
}

void launch_image_charge(const DevMesh &m, const double *phi, const double *ofacets, int32_t n_ofacets, int32_t n_obj,
                         double eps0, double *out, cudaStream_t st) {
    if (n_obj <= 0) return;
    count_launches(1);
    k_image_charge<<<1, 1024, 0, st>>>(m, phi, ofacets, n_ofacets, n_obj, eps0, out);
}

}  // namespace pg
