// Device data layout and kernel launch wrappers of the engine.
//
// Layout in HBM:
//   mesh, per cell: planes [Nc][16] f64 (facet i: c0, nx, ny, nz; one 128-B
//   line per cell), neighbours [Nc] int4 (cell id or -tag), barycentric rows
//   [Nc][12] f64, cell dofs [Nc] int4, DG0 field [Nc] f64x4;
//   per dof: dv_inv, rho accumulator, rho, phi;
//   particles: structure of arrays x, y, z, vx, vy, vz (f64, or f32 in the
//   mixed form), cell (int32, -1 = free slot), species (uint8), id (int64).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pg_screen.h"
#include "punc_gpu.h"

namespace pg {

constexpr int kMaxSpecies = 8;
constexpr int kMaxTags = 256;   // boundary tags: 1 = exterior, 2.. objects (batched runs: one per run)
// Mixed form: the CG1 deposit sums q lambda in int64 units of 2^-kFixedBits
// q_max.  One particle adds at most 2^kFixedBits units to a dof, so a dof's
// sum stays below 2^62 (int64 without overflow, with margin) as long as the
// particle store holds at most kMaxMixedSlots = 2^(62 - kFixedBits) slots,
// whatever the distribution of the particles over the cells.
constexpr int kFixedBits = 30;
constexpr int64_t kMaxMixedSlots = int64_t(1) << (62 - kFixedBits);
constexpr int kDead = -1;                 // cell id of a free particle slot
constexpr int kWalkFail = -2147483647;    // walk step limit reached

struct DevMesh {
    int32_t nc = 0, ndof = 0;
    const double *planes = nullptr;   // [nc][16]
    const int4 *nbr = nullptr;        // [nc]
    const double *bary = nullptr;     // [nc][12]
    const int4 *dofs = nullptr;       // [nc]
    double *E = nullptr;              // [nc][4]
    const double *dv_inv = nullptr;   // [ndof]
    // mixed form: one 64-byte record per cell, {barycentric rows 0-2 in FP32
    // (float4 each), neighbours (int4 bits)}: what the walk, the deposit and
    // the field read, in one aligned pair of sectors; and the FP32 field
    const float4 *cell_f = nullptr;   // [nc][4]
    float *E_f = nullptr;             // [nc][4]
    // CG1 (vertex) field of the ESolver path: [ndof][4] (x, y, z, 0)
    const double *Ev = nullptr;
    const float *Evf = nullptr;
    // point-location bins
    double lo[3] = {0, 0, 0}, bin_h[3] = {1, 1, 1};
    int32_t nbin[3] = {1, 1, 1};
    const int64_t *bin_ptr = nullptr;
    const int32_t *bin_cells = nullptr;
    // point location considers cells in [loc_lo, loc_hi) only (batched runs
    // whose meshes overlap in space)
    int32_t loc_lo = 0, loc_hi = 0x7fffffff;
};

struct DevParticles {
    double *x = nullptr, *y = nullptr, *z = nullptr;
    double *vx = nullptr, *vy = nullptr, *vz = nullptr;
    float *xf = nullptr, *yf = nullptr, *zf = nullptr;
    float *vxf = nullptr, *vyf = nullptr, *vzf = nullptr;
    int32_t *cell = nullptr;
    uint8_t *sp = nullptr;
    int64_t *pid = nullptr;
    int64_t capacity = 0;
    // when set, the number of slots in use is read from device memory (kernels
    // of a captured step: the count changes between replays)
    const int64_t *n_dev = nullptr;
};

// slots in use: the device count when present, else the launch argument
__device__ __forceinline__ int64_t slots_in_use(const DevParticles &p, int64_t n_slots) {
    return p.n_dev ? *p.n_dev : n_slots;
}

// Device-side counters and error word, read back with one copy.
struct DevState {
    int32_t err_code;
    int32_t err_pad;
    int64_t err_index;
    int64_t live[kMaxSpecies];                    // live particles per species
    int64_t absorbed[kMaxTags][kMaxSpecies];      // absorbed this call, per tag and species
    int64_t injected[kMaxSpecies];
    int64_t inject_total;                         // slots appended by the last injection
    int64_t retests;                              // mixed form: facets re-tested in FP64
    double ke;                                    // last kinetic-energy reduction
    double image_charge[kMaxTags];
};

// Per-species constants for one push.
struct PushParams {
    double coef[kMaxSpecies];     // (0.5*dt)*(q/m) for boris, dt*(q/m) for accel
    double half_m[kMaxSpecies];   // 0.5*m
    double t[kMaxSpecies][3];     // Boris rotation vectors (host tan)
    double s[kMaxSpecies][3];
    int32_t has_B;
    int32_t accel;                // 1: accel() update rule
    int32_t cg1;                  // 1: field interpolated from the CG1 vertex field (accel_cg1 / boris_cg1)
    int32_t threads;              // block size of the particle pass (0: 256; at most 512)
};

// EFieldDG0 (punc/src/efield.cpp:95-99) for cell c with barycentric matrix A
// ([12], rows 0-2): E = -(sum_k (phi_k - phi_3) grad lambda_k) + E0, each
// product and sum rounded in this order (the oracle's order, independent of
// the translation unit's --fmad setting).
__device__ __forceinline__ void dg0_field_f64(const double *A, int4 d, const double *phi, double e0x, double e0y,
                                              double e0z, double &ex, double &ey, double &ez) {
    const double p3 = phi[d.w];
    const double a = __dadd_rn(phi[d.x], -p3), b = __dadd_rn(phi[d.y], -p3), e = __dadd_rn(phi[d.z], -p3);
    const double gx = __dadd_rn(__dadd_rn(__dmul_rn(a, A[1]), __dmul_rn(b, A[5])), __dmul_rn(e, A[9]));
    const double gy = __dadd_rn(__dadd_rn(__dmul_rn(a, A[2]), __dmul_rn(b, A[6])), __dmul_rn(e, A[10]));
    const double gz = __dadd_rn(__dadd_rn(__dmul_rn(a, A[3]), __dmul_rn(b, A[7])), __dmul_rn(e, A[11]));
    ex = __dadd_rn(-gx, e0x);
    ey = __dadd_rn(-gy, e0y);
    ez = __dadd_rn(-gz, e0z);
}

struct MoveParams {
    double dt;
    int32_t periodic;
    double Ld[3];
};

struct InjectSpecies {
    double ndt;                   // n*dt
    double domain_lo[3], domain_w[3];
    double vd[3];
    double vth2, factor;
    double q;
};

struct InjectParams {
    int32_t n_species;
    int32_t n_facets;
    uint64_t seed;
    uint32_t step;
    double dt;
    int64_t slot_base;            // first free slot
    int64_t pid_base;
    // when set: slot base, id base and step number read from
    // counts_dev[0], [1], [2] (captured steps)
    const int64_t *counts_dev;
    // when set (batched runs): the stream of facet j is keyed by
    // (seed + facet_seed[j], facet_c1[j]) instead of (seed, j)
    const uint32_t *facet_c1;
    const uint64_t *facet_seed;
    InjectSpecies sp[kMaxSpecies];
    FluxBox32 sp32[kMaxSpecies];  // FP32 screening boxes of sp (flux_box32), built on the host
    // mixed form: exterior facets in FP32, 4 float4 each: (v0, v1.x), (v1.yz,
    // v2.xy), (v2.z, inward normal), (cell as int bits, 0, 0, 0); null in the
    // FP64 form
    const float4 *facets_f;
    // mixed form: fixed-point deposit target and q * 2^kFixedBits / q_max per species
    unsigned long long *rho_fixed;
    float q_scaled[kMaxSpecies];
};

// Mixed-form per-species constants of one particle pass.
struct MixedParams {
    float coef[kMaxSpecies];      // (0.5*dt)*(q/m) or dt*(q/m)
    float half_m[kMaxSpecies];
    float t[kMaxSpecies][3];
    float s[kMaxSpecies][3];
    float q_scaled[kMaxSpecies];  // q * 2^kFixedBits / q_max
    int32_t has_B;
    int32_t accel;
    float dt;
    int32_t periodic;
    float Ld[3];
    int32_t cg1;                  // 1: field interpolated from the CG1 vertex field
    int32_t threads;              // block size of the particle pass (0: 256; at most 512)
    int32_t dep_agg;              // 1: lanes of a warp in the same cell add their deposits before the atomics
    // DG0 field formed in the pass from the potential (when phi is set) at
    // the particle's cell, as dg0_field_f32; else read from the mesh's E_f
    const double *phi;
    float E0[3];
};

// The mixed form's DG0 field of cell c: E = -sum_k phi_k grad lambda_k + E0
// from the cell record's FP32 rows (grad lambda_3 = -(sum of the others)),
// phi differences taken in FP64; explicit fmaf chains, so every translation
// unit forms the same bits.
__device__ __forceinline__ float4 dg0_field_f32(const float4 r0, const float4 r1, const float4 r2, int4 d,
                                                const double *phi, float e0x, float e0y, float e0z) {
    const double p3 = phi[d.w];
    const float a = (float)(phi[d.x] - p3), b = (float)(phi[d.y] - p3), e = (float)(phi[d.z] - p3);
    const float gx = fmaf(e, r2.y, fmaf(b, r1.y, __fmul_rn(a, r0.y)));
    const float gy = fmaf(e, r2.z, fmaf(b, r1.z, __fmul_rn(a, r0.z)));
    const float gz = fmaf(e, r2.w, fmaf(b, r1.w, __fmul_rn(a, r0.w)));
    return make_float4(__fadd_rn(-gx, e0x), __fadd_rn(-gy, e0y), __fadd_rn(-gz, e0z), 0.0f);
}

// ESolver: rhs gather, three-component Jacobi-CG on the mass matrix, packing
// of the vertex field (+ E0).  fp32 selects the FP32 arrays.
struct EsolveArgs {
    int32_t n;                    // dofs
    int32_t fp32;
    const int64_t *adj_ptr;       // dof -> cells, [n + 1]
    const int32_t *adj_cell;
    const double *vol;            // [nc]
    const double *E_cell;         // [nc][4], -grad phi per cell
    const int32_t *row, *col;     // mass matrix CSR
    const double *val, *dinv;
    const float *val32, *dinv32;
    double *b, *x, *r, *z, *p, *Ap;          // [3][n] (FP64 form)
    float *b32, *x32, *r32, *z32, *p32, *Ap32;  // [3][n] (mixed form)
    double *partials;             // [12][grid]
    double rtol, atol;
    int32_t max_iter;
    int32_t *out_iter, *out_status;
    double *out_rr, *out_bb;      // [3] each
    double E0[3];
    double *ev;                   // [n][4] or null
    float *evf;                   // [n][4] or null
};

// PCG on the Dirichlet-reduced symmetric matrix, one cooperative launch.
// The matrix is in SELL-32 form: rows in slices of 32, each slice stored
// column-major (entry k of row 32*s + lane at slice_ptr[s] + 32*k + lane),
// padded to the slice's longest row with (own column, 0.0).
struct PcgArgs {
    int32_t n;
    const int64_t *slice_ptr;     // [n_slices + 1]
    const int32_t *slice_width;   // [n_slices]
    const int32_t *col;
    const double *val;
    const double *dinv;
    double *b;
    double *x;
    double *r;
    double *z;
    double *p0;
    double *p1;
    double *Ap;
    double *partials;             // [4][grid]
    double rtol, atol;
    int32_t max_iter;
    int32_t remove_mean;          // periodic: project b and x onto mean zero
    int32_t *out_iter;
    int32_t *out_status;          // 0 converged, 1 iteration cap, 2 breakdown
    double *out_rr;               // ||r||^2
    double *out_bb;               // ||b||^2
    // mixed solver: FP32 copies of the matrix and the Krylov vectors
    const float *val32;
    const float *dinv32;
    float *r32, *z32, *p32, *Ap32;
    int32_t *out_updates;         // reliable updates done
};

// AMG hierarchy on the device: FP32 sparse operators, each either SELL-32
// (one thread per row, g == 1) or CSR processed by g lanes per row (g a power
// of two: up to 32 within a warp, 64..512 across the warps of one block) for
// operators with long rows.
struct SpOp {
    int32_t n = 0;                       // rows
    int32_t g = 1;                       // lanes per row
    const int64_t *ptr = nullptr;        // SELL slice offsets [n_slices+1] or CSR row offsets [n+1]
    const int32_t *swidth = nullptr;     // SELL slice widths (g == 1 only)
    int32_t wmax = 0;                    // widest SELL slice (g == 1 only)
    const int32_t *col = nullptr;        // column indices (when col16 is null)
    const float *val = nullptr;          // FP32 values (when val16 is null)
    // compressed forms: column = cbase[slice or row] + col16[k]; value =
    // vscale * half(val16[k]) (IEEE binary16 bits)
    const uint16_t *col16 = nullptr;
    const int32_t *cbase = nullptr;
    const uint16_t *val16 = nullptr;
    float vscale = 1.0f;
};

constexpr int kAmgMaxLevels = 12;

struct AmgLevelDev {
    SpOp A;                              // level operator (level 0: the solver's FP32 matrix)
    SpOp ST;                             // S^T to the next level, S = (I - omega D^-1 A) P (not on the last two)
    const float *dinv = nullptr;
    float omega = 0.f;
    float *b = nullptr;                  // right-hand side (levels >= 1)
    float *t = nullptr;                  // W b
};

// The cycle for L = nlev - 1 levels above the coarsest: down-sweep phases
// t_l = W_l b_l with b_{l+1} = S_l^T b_l, the last one y_L = G b_{L-1}
// (G = C^-1 S_{L-1}^T); then y_1 = t_1 + U1 [t_2 .. t_{L-1}, y_L] (L >= 2)
// and z = t_0 + S_0 y_1.  L == 0: z = C^-1 r.
struct AmgDev {
    int32_t nlev = 0;
    AmgLevelDev lev[kAmgMaxLevels];
    SpOp S0, G, U1, cinv;
    float *stack = nullptr;              // [t_2 .. t_{L-1}, y_L] (L >= 2) or y_1 (L == 1)
    float *yL = nullptr;                 // y_L inside the stack
    float *y1 = nullptr;                 // level-1 result (L >= 2)
    float *r_alt = nullptr;              // second FP32 residual buffer of the solver [n]
};

// ---- launch wrappers (all on `stream`) -----------------------------------
int sm_count();
// Kernels launched by this library in this process (pg_launch_count).
void count_launches(int n);
long long launches_so_far();

void launch_efield(const DevMesh &m, const double *phi, const double E0[3], cudaStream_t st);
void launch_push(const DevMesh &m, const DevParticles &p, int64_t n_slots, const PushParams &pp,
                 double *partials, int nblocks, double *ke_out, cudaStream_t st);
void launch_move(const DevParticles &p, int64_t n_slots, const MoveParams &mp, cudaStream_t st);
void launch_update(const DevMesh &m, const DevParticles &p, int64_t n_slots, int max_steps,
                   DevState *state, cudaStream_t st);
void launch_deposit(const DevMesh &m, const DevParticles &p, int64_t n_slots, const double *q_species,
                    double *rho_acc, cudaStream_t st);
void launch_fused_step(const DevMesh &m, const DevParticles &p, int64_t n_slots, const PushParams &pp,
                       const MoveParams &mp, int max_steps, const double *q_species, double *rho_acc,
                       DevState *state, double *partials, int nblocks, double *ke_out, cudaStream_t st);
void launch_kinetic(const DevParticles &p, int64_t n_slots, const double *half_m, double *partials,
                    int nblocks, double *ke_out, cudaStream_t st);
void launch_locate(const DevMesh &m, const double *xyz, int64_t n, int32_t *cells, cudaStream_t st);
void launch_relocate(const DevMesh &m, const double *xyz, const int32_t *start, int64_t n, int mode, int max_steps,
                     int32_t *out, int32_t *cross, cudaStream_t st);
void launch_scale(const double *a, const double *b, double *out, int64_t n, cudaStream_t st);
void launch_extrapolate(double *x, double *x_prev, int64_t n, cudaStream_t st);

void launch_inject_count(const DevMesh &m, const InjectParams &ip, const double *flux_num,
                         int64_t *counts, cudaStream_t st);
void launch_inject_generate(const DevMesh &m, const DevParticles &p, const InjectParams &ip,
                            const double *flux_num, const double *pdf_max, const double *facets,
                            const int64_t *offsets, int max_steps, int deposit, const double *q_species,
                            double *rho_acc, DevState *state, int64_t max_particles, cudaStream_t st);

void launch_scan_i64(const int64_t *in, int64_t *out, int64_t n, int64_t *tmp, cudaStream_t st);
int64_t scan_tmp_size(int64_t n);
void launch_sort_hist(const DevParticles &p, int64_t n_slots, int64_t *hist, cudaStream_t st);
void launch_sort_scatter(const DevParticles &src, const DevParticles &dst, int64_t n_slots,
                         int64_t *cursor, cudaStream_t st);

void launch_rhs(const DevMesh &m, const int64_t *msptr, const int32_t *mswidth, const int32_t *mscol,
                const double *msval, const double *rho, const int32_t *bc_kind, const double *bc_value,
                const double *w_ext, const double *w_obj, const double *obj_pot, int32_t n_obj, int32_t use_ext,
                double *b, cudaStream_t st);
void launch_set_bc(const int32_t *bc_kind, const double *bc_value, const double *obj_pot,
                   int32_t n, double *x, cudaStream_t st);
int launch_pcg(const PcgArgs &a, cudaStream_t st);
int pcg_grid_blocks();
int launch_pcg_amg(const PcgArgs &a, const AmgDev &amg, cudaStream_t st);
int esolve_grid_blocks();
// diagnostics (k_diag.cu)
void launch_potential_energy(const DevMesh &m, const DevParticles &p, int64_t n_slots, bool mixed,
                             const double *qsp, const double *phi, double *out, cudaStream_t st);
void launch_density_cg1(const DevMesh &m, const DevParticles &p, int64_t n_slots, bool mixed, const double *qsp,
                        double we, double wi, double *ne, double *ni, cudaStream_t st);
void launch_density_dg0(const DevMesh &m, const DevParticles &p, int64_t n_slots, const double *qsp,
                        const double *vol, double we, double wi, unsigned long long *cnt, double *ne, double *ni,
                        cudaStream_t st);
void launch_statistics(const DevParticles &p, int64_t n_slots, bool mixed, const double *qsp, double *acc,
                       cudaStream_t st);
int launch_esolve(const EsolveArgs &e, cudaStream_t st);
void launch_pack_ev64(int32_t n, const double *x3, const double E0[3], double *ev, float *evf, cudaStream_t st);
int pcg_amg_grid_blocks();
struct Pots {
    int32_t n;
    double v[kMaxTags];
};
// rng (optional): [2 n_obj] dof range [lo, hi) outside which L_k is dropped
void launch_superpose(const double *phi0, const double *lap, const Pots &pots, const int32_t *rng, int32_t n,
                      double *out, cudaStream_t st);

// CircuitCM matrices and groups on the device (k_step.cu)
struct CircuitDev {
    int32_t n = 0;                       // objects
    int32_t n_groups = 0, n_fv = 0;
    const int32_t *g_ptr = nullptr, *g_mem = nullptr;   // charge-sharing groups
    const int32_t *f_ptr = nullptr, *f_mem = nullptr;   // fixed-voltage sets
    const double *inv_cap = nullptr;     // [n][n]
    const double *inv_circ = nullptr;    // [2n][2n]
    double *cv = nullptr;                // [2n] circuit vector
};
void launch_inject_commit(int64_t *counts, const DevState *st, cudaStream_t s);
void launch_objects_update(const DevState *st, const double *q, int n_species, const int64_t *tags, int n_obj,
                           double *obj, double dt, cudaStream_t s);
void launch_circuit_pre(const double *isrc, int n_isrc, double circ_dt, int n_obj, double *obj, double *obj_pot,
                        cudaStream_t s);
void launch_circuit_post(const CircuitDev &c, const double *img, double *obj, double *obj_pot, cudaStream_t s);
void launch_superpose_dev(const double *phi0, const double *lap, const double *pot, const int32_t *rng, int n_obj,
                         int32_t n, double *out, cudaStream_t s);
void launch_step_record(double *rows, int row_len, int64_t *counts, const double *ke, const DevState *st,
                        int n_species, const int32_t *pcg_i, const double *pcg_d, const double *obj, int n_obj,
                        cudaStream_t s);
void launch_set_count(int64_t *counts, const int64_t *cursor, int32_t nc, cudaStream_t s);

// adjoint of the fused steps (k_adjoint.cu)
void launch_adj_deposit(const DevMesh &m, int64_t n, const int32_t *cell, const uint8_t *sp, const double *q,
                        const double *rhobar, double *xb, double *yb, double *zb, cudaStream_t st);
void launch_adj_move_push(int64_t n, const int32_t *cell, const uint8_t *sp, const double *coef, double dt,
                          const double *xb, const double *yb, const double *zb, double *vxb, double *vyb, double *vzb,
                          double *Ebar, double *e0bar, cudaStream_t st);
void launch_adj_field(const DevMesh &m, const double *Ebar, double *phibar, cudaStream_t st);
void launch_csr_matvec(int32_t n, const int32_t *row, const int32_t *col, const double *val, const double *x,
                       double *y, cudaStream_t st);
void launch_zero_dirichlet(int32_t n, const int32_t *bc_kind, double *v, cudaStream_t st);
void launch_dot_accum(int32_t n, const double *a, const double *b, double *out, cudaStream_t st);
void launch_loss_grad(int32_t n, const double *rho, const double *target, double *rhobar, double *loss,
                      cudaStream_t st);
void launch_scatter_by_id(int64_t n, const int32_t *cell, const int64_t *pid, int64_t pid_base, int64_t n_out,
                          const double *a, const double *b, const double *c, double *out, cudaStream_t st);

// mixed-precision form
void launch_mixed_pass(const DevMesh &m, const DevParticles &p, int64_t n_slots, const MixedParams &mp, bool push,
                       bool move, bool walk, bool deposit, int max_steps, unsigned long long *rho_fixed,
                       DevState *state, double *partials, int nblocks, double *ke_out, cudaStream_t st);
void launch_kinetic_mixed(const DevParticles &p, int64_t n_slots, const MixedParams &mp, double *partials,
                          int nblocks, double *ke_out, cudaStream_t st);
void launch_fixed_to_rho(const unsigned long long *fixed, const double *dv_inv, double unit, int32_t n,
                         double *rho_acc, double *rho, cudaStream_t st);
void launch_float_tables(const double *bary, const int4 *nbr, int32_t nc, float4 *cell_f, cudaStream_t st);
void launch_image_charge(const DevMesh &m, const double *phi, const double *ofacets, int32_t n_ofacets,
                         int32_t n_obj, double eps0, double *out, cudaStream_t st);

}  // namespace pg
