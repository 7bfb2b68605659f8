// Kernels of the adjoint of K fused steps (push, move, deposit, Poisson) in
// the FP64 form, with the cell of each particle fixed from the forward pass
// (the map is piecewise smooth: DG0 field constant per cell, barycentric
// weights linear per cell).  Forward step n:
//   rho_n = dv_inv * sum_p q_p lambda(x_n,p)              (deposit)
//   phi_n = P A^+ P M rho_n                               (P: mean removal on periodic meshes)
//   E_n,c = -sum_k phi_n[d_k] grad lambda_k(c) + E0       (DG0 field)
//   v_n+1/2 = v_n-1/2 + coef_n E_n,c(x_n)                 (accel / boris with B = 0)
//   x_n+1 = x_n + dt v_n+1/2                              (move, periodic wrap)
// Reverse step n, given xbar (for x_n+1) and vbar (for v_n+1/2):
//   vbar += dt xbar;  Ebar_c = sum_{p in c} coef vbar_p;  E0bar += sum Ebar_c
//   phibar[d_k] -= Ebar_c . grad lambda_k(c)
//   rhobar = M P A^+ P phibar      (a second PCG on the same symmetric matrix)
//   xbar += q sum_i dv_inv[d_i] rhobar[d_i] grad lambda_i(c(x_n))
#include <cuda_runtime.h>

#include "pg_device.cuh"

namespace pg {

namespace {

constexpr int kThreads = 256;

// grad lambda_i of cell c (rows 0-2 of the barycentric matrix, lambda_3 = 1 - sum)
__device__ __forceinline__ void grads(const DevMesh &m, int c, double g[4][3]) {
    const double *A = m.bary + 12 * (size_t)c;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) g[i][j] = A[4 * i + 1 + j];
    for (int j = 0; j < 3; ++j) g[3][j] = -(g[0][j] + g[1][j] + g[2][j]);
}

// xbar_p += q_p sum_i dv_inv[d_i] rhobar[d_i] grad lambda_i(c_p)
__global__ void k_adj_deposit(DevMesh m, int64_t n, const int32_t *__restrict__ cell, const uint8_t *__restrict__ sp,
                              const double *__restrict__ q, const double *__restrict__ rhobar, double *__restrict__ xb,
                              double *__restrict__ yb, double *__restrict__ zb) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cell[i];
    if (c < 0) return;
    double g[4][3];
    grads(m, c, g);
    const int4 d = m.dofs[c];
    const int dd[4] = {d.x, d.y, d.z, d.w};
    double s[3] = {0, 0, 0};
    for (int k = 0; k < 4; ++k) {
        const double w = m.dv_inv[dd[k]] * rhobar[dd[k]];
        for (int j = 0; j < 3; ++j) s[j] += w * g[k][j];
    }
    const double qs = q[sp[i]];
    xb[i] += qs * s[0];
    yb[i] += qs * s[1];
    zb[i] += qs * s[2];
}

// vbar += dt xbar; Ebar_c += coef vbar (atomics); E0bar partials
__global__ void k_adj_move_push(int64_t n, const int32_t *__restrict__ cell, const uint8_t *__restrict__ sp,
                                const double *__restrict__ coef, double dt, const double *__restrict__ xb,
                                const double *__restrict__ yb, const double *__restrict__ zb, double *__restrict__ vxb,
                                double *__restrict__ vyb, double *__restrict__ vzb, double *__restrict__ Ebar,
                                double *__restrict__ e0bar) {
    __shared__ double sh[3][kThreads / 32];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double ex = 0, ey = 0, ez = 0;
    if (i < n && cell[i] >= 0) {
        const double vx = vxb[i] + dt * xb[i], vy = vyb[i] + dt * yb[i], vz = vzb[i] + dt * zb[i];
        vxb[i] = vx; vyb[i] = vy; vzb[i] = vz;
        const double k = coef[sp[i]];
        ex = k * vx; ey = k * vy; ez = k * vz;
        const int c = cell[i];
        atomicAdd(Ebar + 3 * (size_t)c, ex);
        atomicAdd(Ebar + 3 * (size_t)c + 1, ey);
        atomicAdd(Ebar + 3 * (size_t)c + 2, ez);
    }
    for (int o = 16; o > 0; o >>= 1) {
        ex += __shfl_down_sync(0xffffffffu, ex, o);
        ey += __shfl_down_sync(0xffffffffu, ey, o);
        ez += __shfl_down_sync(0xffffffffu, ez, o);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sh[0][w] = ex; sh[1][w] = ey; sh[2][w] = ez; }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[threadIdx.x][k];
        atomicAdd(e0bar + threadIdx.x, s);
    }
}

// phibar[d_k] -= Ebar_c . grad lambda_k(c)
__global__ void k_adj_field(DevMesh m, const double *__restrict__ Ebar, double *__restrict__ phibar) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.nc) return;
    const double e[3] = {Ebar[3 * (size_t)c], Ebar[3 * (size_t)c + 1], Ebar[3 * (size_t)c + 2]};
    if (e[0] == 0.0 && e[1] == 0.0 && e[2] == 0.0) return;
    double g[4][3];
    grads(m, c, g);
    const int4 d = m.dofs[c];
    const int dd[4] = {d.x, d.y, d.z, d.w};
    for (int k = 0; k < 4; ++k) atomicAdd(phibar + dd[k], -(e[0] * g[k][0] + e[1] * g[k][1] + e[2] * g[k][2]));
}

// y = M x (CSR), Dirichlet rows of x zeroed first when bc_kind is given
__global__ void k_csr_matvec(int32_t n, const int32_t *__restrict__ row, const int32_t *__restrict__ col,
                             const double *__restrict__ val, const double *__restrict__ x, double *__restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int k = row[i]; k < row[i + 1]; ++k) s = fma(val[k], x[col[k]], s);
    y[i] = s;
}

__global__ void k_zero_dirichlet(int32_t n, const int32_t *__restrict__ bc_kind, double *__restrict__ v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && bc_kind[i] >= 0) v[i] = 0.0;
}

// out += sum_i a_i b_i (block sums, one FP64 atomic per block)
__global__ void k_dot_accum(int32_t n, const double *__restrict__ a, const double *__restrict__ b,
                            double *__restrict__ out) {
    __shared__ double sh[kThreads / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = i < n ? a[i] * b[i] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[k];
        atomicAdd(out, s);
    }
}

// rhobar = 2 (rho - target)
__global__ void k_loss_grad(int32_t n, const double *__restrict__ rho, const double *__restrict__ target,
                            double *__restrict__ rhobar, double *__restrict__ loss) {
    __shared__ double sh[kThreads / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (i < n) {
        const double d = rho[i] - target[i];
        rhobar[i] = 2.0 * d;
        l = d * d;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[k];
        atomicAdd(loss, s);
    }
}

// out[pid - pid_base] = (a, b, c)[slot] for live slots
__global__ void k_scatter_by_id(int64_t n, const int32_t *__restrict__ cell, const int64_t *__restrict__ pid,
                                int64_t pid_base, int64_t n_out, const double *__restrict__ a,
                                const double *__restrict__ b, const double *__restrict__ c, double *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || cell[i] < 0) return;
    const int64_t k = pid[i] - pid_base;
    if (k < 0 || k >= n_out) return;
    out[3 * k] = a[i];
    out[3 * k + 1] = b[i];
    out[3 * k + 2] = c[i];
}

inline unsigned blocks(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

}  // namespace

void launch_adj_deposit(const DevMesh &m, int64_t n, const int32_t *cell, const uint8_t *sp, const double *q,
                        const double *rhobar, double *xb, double *yb, double *zb, cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1);
    k_adj_deposit<<<blocks(n), kThreads, 0, st>>>(m, n, cell, sp, q, rhobar, xb, yb, zb);
}
void launch_adj_move_push(int64_t n, const int32_t *cell, const uint8_t *sp, const double *coef, double dt,
                          const double *xb, const double *yb, const double *zb, double *vxb, double *vyb, double *vzb,
                          double *Ebar, double *e0bar, cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1);
    k_adj_move_push<<<blocks(n), kThreads, 0, st>>>(n, cell, sp, coef, dt, xb, yb, zb, vxb, vyb, vzb, Ebar, e0bar);
}
void launch_adj_field(const DevMesh &m, const double *Ebar, double *phibar, cudaStream_t st) {
    count_launches(1);
    k_adj_field<<<blocks(m.nc), kThreads, 0, st>>>(m, Ebar, phibar);
}
void launch_csr_matvec(int32_t n, const int32_t *row, const int32_t *col, const double *val, const double *x,
                       double *y, cudaStream_t st) {
    count_launches(1);
    k_csr_matvec<<<blocks(n), kThreads, 0, st>>>(n, row, col, val, x, y);
}
void launch_zero_dirichlet(int32_t n, const int32_t *bc_kind, double *v, cudaStream_t st) {
    count_launches(1);
    k_zero_dirichlet<<<blocks(n), kThreads, 0, st>>>(n, bc_kind, v);
}
void launch_dot_accum(int32_t n, const double *a, const double *b, double *out, cudaStream_t st) {
    count_launches(1);
    k_dot_accum<<<blocks(n), kThreads, 0, st>>>(n, a, b, out);
}
void launch_loss_grad(int32_t n, const double *rho, const double *target, double *rhobar, double *loss,
                      cudaStream_t st) {
    count_launches(1);
    k_loss_grad<<<blocks(n), kThreads, 0, st>>>(n, rho, target, rhobar, loss);
}
void launch_scatter_by_id(int64_t n, const int32_t *cell, const int64_t *pid, int64_t pid_base, int64_t n_out,
                          const double *a, const double *b, const double *c, double *out, cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1);
    k_scatter_by_id<<<blocks(n), kThreads, 0, st>>>(n, cell, pid, pid_base, n_out, a, b, c, out);
}

}  // namespace pg
