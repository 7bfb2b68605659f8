// The pg_sim handle: device-resident mesh, particles, fields and solver,
// and the C ABI entry points of punc_gpu.h.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "pg_device.cuh"
#include "pg_reduce.cuh"
#include "pg_amg.h"
#include "pg_internal.h"

using namespace pg;

struct pg_sim {
    pg_config cfg{};
    cudaStream_t stream = nullptr;
    // pg_get_phi_async: a snapshot of phi read back on a copy stream
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t phi_ready = nullptr, phi_copied = nullptr;
    double *phi_snap = nullptr;
    bool phi_copy_pending = false;
    int device = 0;
    std::vector<void *> allocs;  // mesh and solver buffers (freed at destroy)

    // mesh
    DevMesh dm{};
    int32_t nc = 0, ndof = 0, n_obj = 0, n_ext = 0, n_ofac = 0;
    std::vector<double> ext_facets_h, obj_facets_h;
    double *d_ext_facets = nullptr, *d_ofacets = nullptr;
    float4 *d_ext_facets_f = nullptr;     // mixed form: exterior facets in FP32 (InjectParams::facets_f)

    // particles (two buffers for the cell sort)
    DevParticles P[2]{};
    int cur = 0;
    int64_t n_slots = 0, next_pid = 0;
    int n_species = 0;
    double q[kMaxSpecies]{}, m[kMaxSpecies]{};
    double *d_q = nullptr;

    // fields
    double *rho_acc = nullptr, *rho = nullptr, *phi = nullptr, *b = nullptr;
    bool rho_valid = false;
    unsigned long long *rho_fixed = nullptr;   // mixed form: int64 fixed-point accumulator

    // solver
    int64_t *A_sptr = nullptr;                 // SELL-32 slices of the reduced matrix
    int32_t *A_swidth = nullptr, *A_col = nullptr, *M_row = nullptr, *M_col = nullptr;
    double *A_val = nullptr, *A_dinv = nullptr, *M_val = nullptr;
    int64_t *Ms_ptr = nullptr;                           // M in SELL-32 for b = M rho
    int32_t *Ms_width = nullptr, *Ms_col = nullptr;
    double *Ms_val = nullptr;
    double *phi0 = nullptr;                    // zero-potential solution (superposition mode)
    bool phi0_valid = false;
    double *x_prev = nullptr;                  // previous PCG solution (pcg_warm_start == 2)
    const double *x_prev_of = nullptr;         // the solution vector x_prev belongs to
    int x_prev_count = 0;                      // solutions seen for that vector (0, 1, 2+)
    double *lap = nullptr;                     // [n_obj][ndof] unit-potential Laplace solutions
    int32_t *lap_rng = nullptr;                // [n_obj][2] dof range [lo, hi) holding L_k's entries
                                               // above 1e-12 of its largest (a batch run's own dofs)
    int32_t *bc_kind = nullptr;
    double *bc_value = nullptr, *w_ext = nullptr, *w_obj = nullptr;
    double *r = nullptr, *z = nullptr, *p0 = nullptr, *p1 = nullptr, *Ap = nullptr, *pcg_part = nullptr;
    int32_t *pcg_out_i = nullptr;
    double *pcg_out_d = nullptr;
    float *A_val32 = nullptr, *A_dinv32 = nullptr;   // mixed PCG
    float *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *Ap32 = nullptr;
    double *obj_pot = nullptr, *image = nullptr;
    bool has_dirichlet = false;
    bool use_amg = false;                      // AMG-preconditioned mixed PCG
    AmgDev amg{};
    Csr amg_A0;                                // the reduced matrix the hierarchy is built from
    double amg_theta = 0.0;                    // strength threshold of the aggregation
    std::vector<void *> amg_mem;               // device allocations of the hierarchy
    std::vector<void *> *alloc_to = nullptr;   // where dalloc records (null: allocs)
    std::vector<int64_t> amg_rows, amg_nnz, amg_nnz_p;   // per level (pg_poisson_layout_get)
    int64_t a_nnz = 0, a_sell = 0;                       // stored nonzeros and SELL-32 entries of A
    int64_t amg_nnz_g = 0, amg_nnz_u1 = 0;               // cycle operators G and U1
    int64_t amg_cycle_bytes = 0;                        // operator bytes read per AMG-PCG iteration
    // the mixed form's step forms only the FP32 DG0 field; the FP64 one is
    // formed from phi and these E0 when it is asked for
    bool E64_stale = false;
    double E0_last[3] = {0, 0, 0};

    // ESolver (CG1 field): dof -> cell adjacency, cell volumes, mass-matrix
    // D^-1 (and FP32 values), CG work arrays, the packed vertex field
    int64_t *es_adj_ptr = nullptr;
    int32_t *es_adj_cell = nullptr;
    double *es_vol = nullptr, *M_dinv = nullptr, *es_buf = nullptr, *es_part = nullptr, *es_out_d = nullptr;
    float *M_val32 = nullptr, *M_dinv32 = nullptr, *es_buf32 = nullptr;
    int32_t *es_out_i = nullptr;
    double *Ev = nullptr;
    float *Evf = nullptr;

    // multi-step runs (pg_run_steps): device counters [slots, next id, RNG
    // step, result row], objects [n][charge, current, potential, -], tags,
    // current sources, circuit matrices, result rows, captured step graphs
    int64_t *run_counts = nullptr, *run_tags = nullptr;
    double *run_obj = nullptr, *run_isrc = nullptr, *run_rows = nullptr;
    int64_t run_rows_cap = 0;
    CircuitDev circ_dev{};
    bool circ_dev_ready = false;
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};   // one per particle buffer
    std::string graph_key[2];
    int64_t graph_cap[2] = {0, 0};
    long long graph_launches = 0;                          // kernels per captured step

    // adjoint of K fused steps (pg_adjoint_forward / pg_adjoint_backward)
    struct Adjoint {
        bool ready = false;
        int K = 0, C = 0;
        int64_t n = 0;                        // particle slots (fixed over the K steps)
        pg_step_args args{};
        std::vector<pg_object> objects;
        int saved_sort_interval = 0;
        std::vector<void *> mem;              // device allocations of this adjoint
        std::vector<double *> ck_x;           // per checkpoint: x, y, z, vx, vy, vz ([6][n])
        std::vector<int32_t *> ck_c;          // per checkpoint: cells
        double *fin_x = nullptr;              // state after the K steps
        int32_t *fin_c = nullptr;
        int32_t *rec_c = nullptr;             // cells of the steps of one segment ([C][n])
        double *bar = nullptr;                // xbar, ybar, zbar, vxbar, vybar, vzbar ([6][n])
        double *Ebar = nullptr, *phibar = nullptr, *y = nullptr, *rhobar = nullptr, *target = nullptr;
        double *small = nullptr;              // [0..2] E0bar, [3] loss, [8..15] push coefficients
        double *lap = nullptr;                // [n_obj][ndof] unit-potential Laplace solutions L_k
        double *gpot = nullptr;               // [n_obj] sum over steps of <phibar, L_k>
    } adj;

    // diagnostics scratch (allocated on first use)
    double *diag_a = nullptr, *diag_b = nullptr, *diag_acc = nullptr;
    unsigned long long *diag_cnt = nullptr;
    bool phi_valid = false;

    // circuit (capacitance-matrix method)
    bool circuit_ready = false;
    std::vector<double> inv_cap, inv_circ, circ_vec;  // n x n, 2n x 2n, 2n
    std::vector<std::vector<int>> groups;
    std::vector<std::vector<int>> fixed_voltage;
    std::vector<pg_source> vsrc, isrc;
    double circ_dt = 0;

    // injection
    bool flux_ready = false;
    int n_inj_species = 0;
    int inj_sp[kMaxSpecies]{};
    pg_species inj[kMaxSpecies]{};
    double *flux_num = nullptr, *pdf_max = nullptr;
    std::vector<double> flux_num_h;
    std::vector<double> flux_sum_h;            // per injected species: sum over facets of flux_num
    uint32_t *d_inj_c1 = nullptr;              // per exterior facet RNG stream ids (batched runs)
    uint64_t *d_inj_seed = nullptr;            // per exterior facet seed offsets (batched runs)
    int64_t *inj_counts = nullptr, *inj_offsets = nullptr, *scan_tmp = nullptr;
    int64_t scan_tmp_n = 0;

    // reductions, state
    DevState *state = nullptr;
    DevState *state_h = nullptr;   // pinned
    double *partials = nullptr, *ke_dev = nullptr;
    int n_part = 0;                           // blocks of a particle pass (partial sums in use)
    int part_cap = 0;                         // partial-sum slots allocated
    int32_t tune_threads = 0;                 // particle-pass block size (0: 256)
    int32_t tune_dep_agg = 0;                 // warp-aggregated fixed-point deposit

    // sort scratch
    int64_t *sort_hist = nullptr, *sort_cursor = nullptr;

    // profiling
    bool profiling = false;
    std::vector<std::string> stage_names;
    std::vector<double> stage_ms;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    cudaEvent_t user_ev[16]{};
    int64_t step_count = 0;
};

namespace {

#define PG_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(PG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
    } while (0)

template <class T>
int dalloc(pg_sim *s, T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T));
    if (e != cudaSuccess) return fail(PG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    (s->alloc_to ? *s->alloc_to : s->allocs).push_back(q);
    *p = reinterpret_cast<T *>(q);
    return PG_OK;
}

template <class T>
int upload(pg_sim *s, T **p, const std::vector<T> &h) {
    int rc = dalloc(s, p, h.size());
    if (rc) return rc;
    if (!h.empty()) PG_CUDA(cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return PG_OK;
}

static std::string mixed_capacity_message(int64_t slots) {
    return "the mixed form holds at most " + std::to_string(kMaxMixedSlots) + " particle slots (int64 deposit sums in "
           "units of 2^-" + std::to_string(kFixedBits) + " q_max cannot overflow below that); " +
           std::to_string(slots) + " requested";
}

void free_particles(DevParticles &p) {
    void *ptrs[] = {p.x, p.y, p.z, p.vx, p.vy, p.vz, p.xf, p.yf, p.zf, p.vxf, p.vyf, p.vzf, p.cell, p.sp, p.pid};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    p = DevParticles{};
}

int alloc_particles(pg_sim *s, DevParticles &p, int64_t cap) {
    p = DevParticles{};
    if (s->cfg.precision == PG_MIXED && cap > kMaxMixedSlots)
        return fail(PG_ERR_CAPACITY, mixed_capacity_message(cap));
    p.capacity = cap;
    auto al = [&](void **q, size_t bytes) -> bool { return cudaMalloc(q, bytes) == cudaSuccess; };
    bool ok = true;
    const size_t n = (size_t)cap;
    if (s->cfg.precision == PG_MIXED) {
        ok &= al((void **)&p.xf, n * 4) && al((void **)&p.yf, n * 4) && al((void **)&p.zf, n * 4);
        ok &= al((void **)&p.vxf, n * 4) && al((void **)&p.vyf, n * 4) && al((void **)&p.vzf, n * 4);
    } else {
        ok &= al((void **)&p.x, n * 8) && al((void **)&p.y, n * 8) && al((void **)&p.z, n * 8);
        ok &= al((void **)&p.vx, n * 8) && al((void **)&p.vy, n * 8) && al((void **)&p.vz, n * 8);
    }
    ok &= al((void **)&p.cell, n * 4) && al((void **)&p.sp, n) && al((void **)&p.pid, n * 8);
    if (!ok) {
        free_particles(p);
        return fail(PG_ERR_CUDA, "cudaMalloc: particle store of " + std::to_string(cap) + " slots");
    }
    return PG_OK;
}

int copy_particles(pg_sim *s, const DevParticles &src, const DevParticles &dst, int64_t n) {
    if (n <= 0) return PG_OK;
    auto cp = [&](void *d, const void *q, size_t bytes) {
        return cudaMemcpyAsync(d, q, bytes, cudaMemcpyDeviceToDevice, s->stream);
    };
    if (s->cfg.precision == PG_MIXED) {
        PG_CUDA(cp(dst.xf, src.xf, n * 4)); PG_CUDA(cp(dst.yf, src.yf, n * 4)); PG_CUDA(cp(dst.zf, src.zf, n * 4));
        PG_CUDA(cp(dst.vxf, src.vxf, n * 4)); PG_CUDA(cp(dst.vyf, src.vyf, n * 4)); PG_CUDA(cp(dst.vzf, src.vzf, n * 4));
    } else {
        PG_CUDA(cp(dst.x, src.x, n * 8)); PG_CUDA(cp(dst.y, src.y, n * 8)); PG_CUDA(cp(dst.z, src.z, n * 8));
        PG_CUDA(cp(dst.vx, src.vx, n * 8)); PG_CUDA(cp(dst.vy, src.vy, n * 8)); PG_CUDA(cp(dst.vz, src.vz, n * 8));
    }
    PG_CUDA(cp(dst.cell, src.cell, n * 4));
    PG_CUDA(cp(dst.sp, src.sp, n));
    PG_CUDA(cp(dst.pid, src.pid, n * 8));
    return PG_OK;
}

// Grow both particle buffers to hold `need` slots.
int ensure_capacity(pg_sim *s, int64_t need) {
    if (need <= s->P[0].capacity) return PG_OK;
    int64_t cap = std::max<int64_t>(need + need / 2, std::max<int64_t>(2 * s->P[0].capacity, 1 << 16));
    if (s->cfg.precision == PG_MIXED) {
        if (need > kMaxMixedSlots) return fail(PG_ERR_CAPACITY, mixed_capacity_message(need));
        cap = std::min(cap, kMaxMixedSlots);
    }
    for (int k = 0; k < 2; ++k) {
        DevParticles np;
        int rc = alloc_particles(s, np, cap);
        if (rc) return rc;
        if (k == s->cur) {
            rc = copy_particles(s, s->P[k], np, s->n_slots);
            if (rc) { free_particles(np); return rc; }
            PG_CUDA(cudaStreamSynchronize(s->stream));
        }
        free_particles(s->P[k]);
        s->P[k] = np;
    }
    return PG_OK;
}

int check_state(pg_sim *s) {
    PG_CUDA(cudaMemcpyAsync(s->state_h, s->state, sizeof(DevState), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    if (s->state_h->err_code != 0) {
        // report once, then clear the device error word so the handle stays usable
        const int code = s->state_h->err_code;
        const int64_t idx = s->state_h->err_index;
        cudaMemsetAsync(s->state, 0, 2 * sizeof(int64_t), s->stream);
        cudaStreamSynchronize(s->stream);
        s->state_h->err_code = 0;
        s->state_h->err_index = 0;
        return fail(code, "device error " + std::to_string(code) + " at index " + std::to_string(idx));
    }
    return PG_OK;
}

int species_id(pg_sim *s, double q, double m) {
    for (int k = 0; k < s->n_species; ++k)
        if (s->q[k] == q && s->m[k] == m) return k;
    if (s->n_species >= kMaxSpecies) return -1;
    const int k = s->n_species++;
    s->q[k] = q;
    s->m[k] = m;
    cudaMemcpyAsync(s->d_q, s->q, sizeof(double) * kMaxSpecies, cudaMemcpyHostToDevice, s->stream);
    return k;
}

void stage_begin(pg_sim *s, const char *name, cudaEvent_t *out_end) {
    *out_end = nullptr;
    if (!s->profiling) return;
    int id = -1;
    for (size_t k = 0; k < s->stage_names.size(); ++k)
        if (s->stage_names[k] == name) id = (int)k;
    if (id < 0) {
        s->stage_names.push_back(name);
        s->stage_ms.push_back(0.0);
        id = (int)s->stage_names.size() - 1;
    }
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s->stream);
    s->ev_pending.push_back({id, {a, b}});
    *out_end = b;
}

void stage_end(pg_sim *s, cudaEvent_t end) {
    if (end) cudaEventRecord(end, s->stream);
}

void collect_stages(pg_sim *s) {
    if (s->ev_pending.empty()) return;
    cudaStreamSynchronize(s->stream);
    for (auto &e : s->ev_pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e.second.first, e.second.second);
        s->stage_ms[e.first] += ms;
        cudaEventDestroy(e.second.first);
        cudaEventDestroy(e.second.second);
    }
    s->ev_pending.clear();
}

struct StageScope {
    pg_sim *s;
    cudaEvent_t end;
    StageScope(pg_sim *s_, const char *n) : s(s_) { stage_begin(s, n, &end); }
    ~StageScope() { stage_end(s, end); }
};

// ---- circuit (capacitance-matrix method) ---------------------------------

// In-place inverse by Gauss-Jordan elimination with partial pivoting.
bool invert(std::vector<double> &a, int n) {
    std::vector<double> inv(n * n, 0.0);
    for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c])) piv = r;
        if (a[piv * n + c] == 0.0) return false;
        if (piv != c)
            for (int k = 0; k < n; ++k) { std::swap(a[c * n + k], a[piv * n + k]); std::swap(inv[c * n + k], inv[piv * n + k]); }
        const double d = a[c * n + c];
        for (int k = 0; k < n; ++k) { a[c * n + k] /= d; inv[c * n + k] /= d; }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = a[r * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) { a[r * n + k] -= f * a[c * n + k]; inv[r * n + k] -= f * inv[c * n + k]; }
        }
    }
    a = inv;
    return true;
}

// Charge-sharing sets: objects joined by voltage sources
// (get_charge_sharing_sets, punc/src/object.cpp:80-135).
void collect_group(std::vector<pg_source> &vs, int node, std::vector<int> &group) {
    group.push_back(node);
    size_t i = 0;
    while (i < vs.size()) {
        const pg_source v = vs[i];
        if (v.node_a == node) { vs.erase(vs.begin() + i); collect_group(vs, v.node_b, group); }
        else if (v.node_b == node) { vs.erase(vs.begin() + i); collect_group(vs, v.node_a, group); }
        else ++i;
    }
}

std::vector<std::vector<int>> charge_sharing_sets(std::vector<pg_source> vs, int n_obj) {
    std::vector<int> nodes(n_obj);
    for (int i = 0; i < n_obj; ++i) nodes[i] = i;
    std::vector<std::vector<int>> groups;
    while (!vs.empty()) {
        std::vector<int> g;
        collect_group(vs, vs[0].node_a, g);
        groups.push_back(g);
    }
    for (auto &g : groups)
        for (int v : g)
            if (v != -1) nodes.erase(std::remove(nodes.begin(), nodes.end(), v), nodes.end());
    groups.erase(std::remove_if(groups.begin(), groups.end(),
                                [](const std::vector<int> &g) { return std::find(g.begin(), g.end(), -1) != g.end(); }),
                 groups.end());
    for (int v : nodes) groups.push_back({v});
    return groups;
}

}  // namespace

// ---- solver internals ------------------------------------------------------

// Lanes per row of an AMG operator: SELL-32 with one thread per row up to 12
// entries a row on average, else CSR with a power of two of lanes (at most
// 512, the block) giving each lane three to six entries.
// Lanes per row for an operator applied by `threads` threads of the
// cooperative PCG: the choice with the shortest chain of dependent memory
// round trips per thread, the quantity that bounds a latency-bound phase.
// g == 1: SELL-32, one thread per row, four rows and two entries of each per
// step; g = 2..32: CSR, g lanes per row, four rows per lane group, two entries
// per lane per step; g = 64..512: the warps of one block per row, four
// entries per lane per step.  A round (rows of one pass) costs one trip for
// the row offsets plus two (column, then value gathered) per step.
static int lanes_per_row(const Csr &A, int64_t threads) {
    const double n = (double)std::max<int64_t>(1, A.n);
    double avg = A.n > 0 ? (double)A.ci.size() / n : 0.0, wmax = 0.0;
    for (int64_t r = 0; r < A.n; ++r) wmax = std::max(wmax, (double)(A.rp[r + 1] - A.rp[r]));
    const double T = (double)std::max<int64_t>(threads, 32);
    auto chain = [&](int g) {
        if (g == 1) {
            // SELL slices pad to their longest row
            const double rounds = std::ceil(n / T / 4.0), steps = std::ceil(std::min(wmax, 1.25 * avg) / 2.0);
            return rounds * (1.0 + 2.0 * steps);
        }
        if (g <= 32) {
            const double groups = std::floor(T / g), rounds = std::ceil(n / groups / 4.0);
            return rounds * (1.0 + 2.0 * std::ceil(avg / g / 2.0));
        }
        const double per_round = std::floor(T / g), rounds = std::ceil(n / per_round);
        return rounds * (2.0 + 2.0 * std::ceil(avg / g / 4.0));   // + the block's partial-sum barriers
    };
    int best = avg <= 12.0 ? 1 : 2;
    double bc = chain(best);
    for (int g = 2; g <= 512; g *= 2) {
        const double c = chain(g);
        if (c < bc - 1e-9) { bc = c; best = g; }
    }
    return best;
}

// Upload a CSR operator: SELL-32 (padding: the slice's first column, value
// 0) when g == 1, else CSR.  c16: 16-bit column offsets from the smallest
// column of each slice (SELL) or row (CSR), when every span fits in 16 bits;
// v16: IEEE binary16 values of v / vscale with vscale = max|v| / 1024 (the
// preconditioner's operators; binary16 keeps 11 significant bits, and halving
// the bytes keeps the hierarchy of large meshes resident in L2).
static int upload_op(pg_sim *s, const Csr &A, int g, SpOp &out, bool want_c16 = false, bool want_v16 = false) {
    const int64_t n = A.n;
    int rc;
    out = SpOp{};
    out.n = (int32_t)n;
    out.g = g;
    std::vector<int64_t> ptr;     // slice or row offsets
    std::vector<int32_t> swidth;
    std::vector<int32_t> col;
    std::vector<double> val;
    std::vector<int32_t> base;    // smallest column per slice or row
    if (g > 1) {
        ptr.assign(A.rp.begin(), A.rp.end());
        col.assign(A.ci.begin(), A.ci.end());
        val.assign(A.v.begin(), A.v.end());
        base.assign(n, 0);
        for (int64_t r = 0; r < n; ++r)
            if (A.rp[r + 1] > A.rp[r]) base[r] = *std::min_element(A.ci.begin() + A.rp[r], A.ci.begin() + A.rp[r + 1]);
    } else {
        const int64_t nsl = (n + 31) / 32;
        ptr.assign(nsl + 1, 0);
        swidth.assign(nsl, 0);
        base.assign(nsl, 0);
        for (int64_t sl = 0; sl < nsl; ++sl) {
            int64_t w = 0;
            int32_t b = INT32_MAX;
            for (int64_t r = 32 * sl; r < std::min(n, 32 * sl + 32); ++r) {
                w = std::max(w, A.rp[r + 1] - A.rp[r]);
                for (int64_t k = A.rp[r]; k < A.rp[r + 1]; ++k) b = std::min(b, A.ci[k]);
            }
            swidth[sl] = (int32_t)w;
            base[sl] = b == INT32_MAX ? 0 : b;
            ptr[sl + 1] = ptr[sl] + 32 * w;
        }
        col.assign(std::max<int64_t>(1, ptr[nsl]), 0);
        val.assign(std::max<int64_t>(1, ptr[nsl]), 0.0);
        for (int64_t sl = 0; sl < nsl; ++sl)
            for (int64_t o = ptr[sl]; o < ptr[sl + 1]; ++o) col[o] = base[sl];
        for (int64_t sl = 0; sl < nsl; ++sl)
            for (int lane = 0; lane < 32; ++lane) {
                const int64_t r = 32 * sl + lane;
                if (r >= n) continue;
                const int64_t len = A.rp[r + 1] - A.rp[r];
                for (int64_t k = 0; k < len; ++k) {
                    const int64_t o = ptr[sl] + 32 * k + lane;
                    col[o] = A.ci[A.rp[r] + k];
                    val[o] = A.v[A.rp[r] + k];
                }
            }
    }
    if (ptr.back() > (int64_t)INT32_MAX) return fail(PG_ERR_ARG, "operator with 2^31 or more stored entries");
    if (col.empty()) col.push_back(0);
    if (val.empty()) val.push_back(0.0);
    bool c16 = want_c16;
    if (c16) {
        const int64_t units = (int64_t)base.size();
        for (int64_t u = 0; u < units && c16; ++u)
            for (int64_t o = ptr[u]; o < ptr[u + 1]; ++o)
                if ((int64_t)col[o] - base[u] > 65535) { c16 = false; break; }
    }
    int64_t *d_ptr;
    if ((rc = upload(s, &d_ptr, ptr))) return rc;
    out.ptr = d_ptr;
    if (g == 1) {
        int32_t *d_sw;
        if ((rc = upload(s, &d_sw, swidth))) return rc;
        out.swidth = d_sw;
        out.wmax = swidth.empty() ? 0 : *std::max_element(swidth.begin(), swidth.end());
    }
    if (c16) {
        std::vector<uint16_t> c(col.size(), 0);
        const int64_t units = (int64_t)base.size();
        for (int64_t u = 0; u < units; ++u)
            for (int64_t o = ptr[u]; o < ptr[u + 1]; ++o) c[o] = (uint16_t)(col[o] - base[u]);
        uint16_t *d_c;
        int32_t *d_b;
        if ((rc = upload(s, &d_c, c)) || (rc = upload(s, &d_b, base))) return rc;
        out.col16 = d_c;
        out.cbase = d_b;
    } else {
        int32_t *d_col;
        if ((rc = upload(s, &d_col, col))) return rc;
        out.col = d_col;
    }
    if (want_v16) {
        double vmax = 0.0;
        for (double v : val) vmax = std::max(vmax, std::fabs(v));
        const double sc = vmax > 0.0 ? vmax / 1024.0 : 1.0;
        std::vector<uint16_t> h(val.size());
        for (size_t k = 0; k < val.size(); ++k) h[k] = __half_as_ushort(__float2half_rn((float)(val[k] / sc)));
        uint16_t *d_h;
        if ((rc = upload(s, &d_h, h))) return rc;
        out.val16 = d_h;
        out.vscale = (float)sc;
    } else {
        std::vector<float> v32(val.begin(), val.end());
        float *d_val;
        if ((rc = upload(s, &d_val, v32))) return rc;
        out.val = d_val;
    }
    return PG_OK;
}

// Smoothed-aggregation hierarchy of the reduced Poisson matrix s->amg_A0
// with strength threshold s->amg_theta, on the device, with the operators of
// the collapsed cycle.  Level 0 shares the solver's D^-1.  Device memory goes
// to s->amg_mem (freed by a rebuild).
static int build_amg(pg_sim *s) {
    const Csr &A0 = s->amg_A0;
    AmgHierarchy h;
    AmgParams prm;
    prm.theta = s->amg_theta;
    const int arc = amg_setup(A0, h, s->cfg.periodic != 0, prm);
    if (arc == 9) return fail(PG_ERR_ARG, "AMG: coarsening stalls above 4096 rows (use pcg_precond = 1)");
    if (arc != 0) return fail(PG_ERR_SINGULAR, "AMG: coarsest operator is singular");
    if ((int)h.levels.size() > kAmgMaxLevels) return fail(PG_ERR_ARG, "AMG: too many levels");
    AmgCycle cyc;
    amg_cycle_operators(h, cyc);
    s->amg_nnz_g = (int64_t)cyc.G.ci.size();
    s->amg_nnz_u1 = (int64_t)cyc.U1.ci.size();
    AmgDev &M = s->amg;
    M = AmgDev{};
    // threads of the solve's grid (fewer blocks for small systems)
    const int64_t gt = (int64_t)std::min<int64_t>(pcg_amg_grid_blocks(), (A0.n + kPcgThreads - 1) / kPcgThreads) *
                       kPcgThreads;
    M.nlev = (int32_t)h.levels.size();
    const int L = M.nlev - 1;
    s->amg_rows.assign(M.nlev, 0);
    s->amg_nnz.assign(M.nlev, 0);
    s->amg_nnz_p.assign(M.nlev, 0);
    int rc;
    if (L >= 1 && (rc = dalloc(s, &M.stack, cyc.stack_len))) return rc;
    if ((rc = dalloc(s, &M.r_alt, h.levels[0].A.n))) return rc;
    for (int l = 0; l < M.nlev; ++l) {
        const AmgLevel &Lv = h.levels[l];
        s->amg_rows[l] = Lv.A.n;
        s->amg_nnz[l] = (int64_t)Lv.A.ci.size();
        if (l < L) s->amg_nnz_p[l] = (int64_t)Lv.S.ci.size();
        AmgLevelDev &D = M.lev[l];
        if (l == 0) {
            // the PCG's own product A p reads level 0's operator, also when
            // L == 0: FP32 values (the Krylov recurrence), 16-bit columns
            if ((rc = upload_op(s, Lv.A, 1, D.A, true, false))) return rc;
            D.dinv = s->A_dinv32;
        }
        if (l == L) break;   // the coarsest level lives in G (or cinv when L == 0)
        if (l > 0) {
            if ((rc = upload_op(s, Lv.A, lanes_per_row(Lv.A, gt), D.A, true, true))) return rc;
            std::vector<float> dinv(Lv.dinv.begin(), Lv.dinv.end());
            float *d_dinv;
            if ((rc = upload(s, &d_dinv, dinv)) || (rc = dalloc(s, &D.b, Lv.A.n))) return rc;
            D.dinv = d_dinv;
        }
        D.omega = (float)Lv.omega;
        if (l < L - 1 && (rc = upload_op(s, Lv.ST, lanes_per_row(Lv.ST, gt), D.ST, true, true))) return rc;
        if (l >= 2) D.t = M.stack + cyc.stack_off[l];
        else if ((rc = dalloc(s, &D.t, Lv.A.n))) return rc;
    }
    if (L == 0) {
        // the whole operator is the coarsest: z = C^-1 r
        const int64_t nc = h.levels[0].A.n;
        Csr C;
        C.n = C.m = nc;
        C.rp.resize(nc + 1);
        C.ci.resize(nc * nc);
        for (int64_t i = 0; i <= nc; ++i) C.rp[i] = i * nc;
        for (int64_t k = 0; k < nc * nc; ++k) C.ci[k] = (int32_t)(k % nc);
        C.v = h.coarse_inv;
        if ((rc = upload_op(s, C, lanes_per_row(C, gt), M.cinv))) return rc;
    } else {
        if ((rc = upload_op(s, h.levels[0].S, lanes_per_row(h.levels[0].S, gt), M.S0, true, true)) ||
            (rc = upload_op(s, cyc.G, lanes_per_row(cyc.G, gt), M.G)))
            return rc;
        M.yL = L >= 2 ? M.stack + cyc.stack_off[L] : M.stack;
        if (L >= 2 && ((rc = upload_op(s, cyc.U1, lanes_per_row(cyc.U1, gt), M.U1, true, true)) ||
                       (rc = dalloc(s, &M.y1, h.levels[1].A.n))))
            return rc;
    }
    // the solver kernel takes each operator's value format from its role:
    // binary16 for the preconditioner's transfer and coarse operators, FP32
    // for A_0, G and the coarsest inverse
    bool fmt = M.lev[0].A.val16 == nullptr;
    for (int l = 1; l < L; ++l) fmt = fmt && M.lev[l].A.val16 != nullptr;
    for (int l = 0; l + 1 < L; ++l) fmt = fmt && M.lev[l].ST.val16 != nullptr;
    if (L >= 1) fmt = fmt && M.S0.val16 != nullptr && M.G.val16 == nullptr;
    if (L >= 2) fmt = fmt && M.U1.val16 != nullptr;
    if (L == 0) fmt = fmt && M.cinv.val16 == nullptr;
    if (!fmt) return fail(PG_ERR_ARG, "AMG: operator value formats differ from the solver's");
    // operator bytes of one iteration: A_0 twice (A p and the level-0
    // smoother), then each operator of the cycle once
    auto opb = [](const SpOp &o, int64_t entries) {
        return entries * ((o.col16 ? 2 : 4) + (o.val16 ? 2 : 4));
    };
    int64_t cb = 2 * opb(M.lev[0].A, (int64_t)h.levels[0].A.ci.size());
    if (L == 0) {
        cb += opb(M.cinv, h.levels[0].A.n * h.levels[0].A.n);
    } else {
        cb += opb(M.S0, (int64_t)h.levels[0].S.ci.size());
        if (L >= 2) cb += opb(M.lev[0].ST, (int64_t)h.levels[0].ST.ci.size());
        for (int l = 1; l < L; ++l) {
            cb += opb(M.lev[l].A, (int64_t)h.levels[l].A.ci.size());
            if (l < L - 1) cb += opb(M.lev[l].ST, (int64_t)h.levels[l].ST.ci.size());
        }
        cb += opb(M.G, (int64_t)cyc.G.ci.size());
        if (L >= 2) cb += opb(M.U1, (int64_t)cyc.U1.ci.size());
    }
    s->amg_cycle_bytes = cb;
    s->use_amg = true;
    return PG_OK;
}

static void free_amg(pg_sim *s) {
    for (void *p : s->amg_mem) cudaFree(p);
    s->amg_mem.clear();
    s->amg = AmgDev{};
    s->use_amg = false;
}

static int rebuild_amg(pg_sim *s) {
    free_amg(s);
    s->alloc_to = &s->amg_mem;
    const int rc = build_amg(s);
    s->alloc_to = nullptr;
    return rc;
}

static int setup_amg(pg_sim *s, const std::vector<int32_t> &arow, const std::vector<int32_t> &acol,
                     const std::vector<double> &aval) {
    Csr &A0 = s->amg_A0;
    A0.n = A0.m = (int64_t)arow.size() - 1;
    A0.rp.assign(arow.begin(), arow.end());
    A0.ci = acol;
    A0.v = aval;
    return rebuild_amg(s);
}

static int object_index(const pg_sim *s, int64_t bnd_id) {
    const int64_t k = bnd_id - 2;
    return (k >= 0 && k < s->n_obj) ? (int)k : -1;
}

// One Poisson solve with the given object potentials into x (s->phi unless
// given); rho from s->rho or zero; warm start from x's previous content when
// `warm` and configured.
static int poisson_solve_internal(pg_sim *s, const double *pot_h, bool zero_rho, bool use_ext, double rtol,
                                  double atol, pg_solve_info *acc, double *x_target = nullptr, bool *warm = nullptr) {
    if (s->n_obj > 0) PG_CUDA(cudaMemcpyAsync(s->obj_pot, pot_h, sizeof(double) * s->n_obj, cudaMemcpyHostToDevice, s->stream));
    if (zero_rho) PG_CUDA(cudaMemsetAsync(s->rho_acc, 0, sizeof(double) * s->ndof, s->stream));
    launch_rhs(s->dm, s->Ms_ptr, s->Ms_width, s->Ms_col, s->Ms_val, zero_rho ? s->rho_acc : s->rho, s->bc_kind, s->bc_value, s->w_ext,
               s->w_obj, s->obj_pot, s->n_obj, use_ext ? 1 : 0, s->b, s->stream);
    if (zero_rho) s->rho_valid = false;
    double *x = x_target ? x_target : s->phi;
    bool *valid = warm ? warm : &s->phi_valid;
    if (!(s->cfg.pcg_warm_start && *valid) || zero_rho) {
        PG_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * s->ndof, s->stream));
        if (s->x_prev_of == x) s->x_prev_count = 0;
    } else if (s->cfg.pcg_warm_start == 2) {
        // start from the linear extrapolation of the last two solutions
        if (!s->x_prev) {
            int rc = dalloc(s, &s->x_prev, s->ndof);
            if (rc) return rc;
        }
        if (s->x_prev_of != x) { s->x_prev_of = x; s->x_prev_count = 0; }
        if (s->x_prev_count >= 1) launch_extrapolate(x, s->x_prev, s->ndof, s->stream);
        else PG_CUDA(cudaMemcpyAsync(s->x_prev, x, sizeof(double) * s->ndof, cudaMemcpyDeviceToDevice, s->stream));
        ++s->x_prev_count;
    }
    launch_set_bc(s->bc_kind, use_ext ? s->bc_value : nullptr, s->obj_pot, s->ndof, x, s->stream);
    PcgArgs a{};
    a.n = s->ndof;
    a.slice_ptr = s->A_sptr; a.slice_width = s->A_swidth; a.col = s->A_col; a.val = s->A_val; a.dinv = s->A_dinv;
    a.b = s->b; a.x = x; a.r = s->r; a.z = s->z; a.p0 = s->p0; a.p1 = s->p1; a.Ap = s->Ap;
    a.partials = s->pcg_part;
    a.rtol = rtol; a.atol = atol;
    a.max_iter = s->cfg.pcg_max_iter;
    a.remove_mean = s->cfg.periodic ? 1 : 0;
    a.out_iter = s->pcg_out_i; a.out_status = s->pcg_out_i + 1;
    a.out_rr = s->pcg_out_d; a.out_bb = s->pcg_out_d + 1;
    a.val32 = s->A_val32; a.dinv32 = s->A_dinv32;
    a.r32 = s->r32; a.z32 = s->z32; a.p32 = s->p32; a.Ap32 = s->Ap32;
    a.out_updates = nullptr;
    int e;
    {
        StageScope t(s, "pcg");
        e = s->use_amg ? launch_pcg_amg(a, s->amg, s->stream) : launch_pcg(a, s->stream);
    }
    if (e) return fail(PG_ERR_CUDA, std::string("cooperative PCG launch: ") + cudaGetErrorString((cudaError_t)e));
    int32_t oi[2];
    double od[2];
    PG_CUDA(cudaMemcpyAsync(oi, s->pcg_out_i, sizeof(oi), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaMemcpyAsync(od, s->pcg_out_d, sizeof(od), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    *valid = true;
    if (acc) {
        acc->iterations += oi[0];
        acc->solves += 1;
        acc->residual = std::sqrt(od[0]);
        acc->rhs_norm = std::sqrt(od[1]);
    }
    if (oi[1] == 1) return fail(PG_ERR_NOT_CONVERGED, "PCG reached " + std::to_string(oi[0]) + " iterations, ||r|| = " + std::to_string(std::sqrt(od[0])));
    if (oi[1] == 2) return fail(PG_ERR_NOT_CONVERGED, "PCG breakdown (p.Ap <= 0) at iteration " + std::to_string(oi[0]));
    if (oi[1] == 3)
        return fail(PG_ERR_NOT_CONVERGED, "PCG stalled at ||r|| = " + std::to_string(std::sqrt(od[0])) + " after " +
                                              std::to_string(oi[0]) + " iterations: the tolerance is below the "
                                              "attainable accuracy of the mixed-precision recurrence");
    return PG_OK;
}

static int image_charges(pg_sim *s, std::vector<double> &out, const double *phi = nullptr) {
    out.assign(s->n_obj, 0.0);
    if (s->n_obj == 0) return PG_OK;
    launch_image_charge(s->dm, phi ? phi : s->phi, s->d_ofacets, s->n_ofac, s->n_obj, s->cfg.eps0, s->image, s->stream);
    PG_CUDA(cudaMemcpyAsync(out.data(), s->image, sizeof(double) * s->n_obj, cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return PG_OK;
}

static bool is_mixed(const pg_sim *s) { return s->cfg.precision == PG_MIXED; }

// Fixed-point unit of the mixed deposit: 2^-kFixedBits of the largest |q|
// (the store limit kMaxMixedSlots keeps every dof's int64 sum below 2^62).
static double fixed_unit(const pg_sim *s) {
    double qmax = 0.0;
    for (int k = 0; k < s->n_species; ++k) qmax = std::max(qmax, std::fabs(s->q[k]));
    if (qmax == 0.0) qmax = 1.0;
    return std::ldexp(qmax, -kFixedBits);
}

static void fill_mixed(const pg_sim *s, MixedParams &mp, double dt_push, const double *B, bool accel, double dt_move,
                       bool periodic, const double *Ld) {
    mp = MixedParams{};
    mp.accel = accel ? 1 : 0;
    mp.has_B = (!accel && B && (B[0] != 0.0 || B[1] != 0.0 || B[2] != 0.0)) ? 1 : 0;
    const double unit = fixed_unit(s);
    for (int k = 0; k < s->n_species; ++k) {
        const double q = s->q[k], m = s->m[k];
        mp.coef[k] = (float)(accel ? dt_push * (q / m) : 0.5 * dt_push * (q / m));
        mp.half_m[k] = (float)(0.5 * m);
        mp.q_scaled[k] = (float)(q / unit);
        if (mp.has_B) {
            double t[3], t2 = 0.0;
            for (int i = 0; i < 3; ++i) { t[i] = std::tan((dt_push * q / (2.0 * m)) * B[i]); t2 += t[i] * t[i]; }
            for (int i = 0; i < 3; ++i) { mp.t[k][i] = (float)t[i]; mp.s[k][i] = (float)(2 * t[i] / (1 + t2)); }
        }
    }
    mp.dt = (float)dt_move;
    mp.periodic = periodic ? 1 : 0;
    mp.threads = s->tune_threads;
    mp.dep_agg = s->tune_dep_agg;
    for (int j = 0; j < 3; ++j) mp.Ld[j] = Ld ? (float)Ld[j] : 1.0f;
}

static int rho_from_acc(pg_sim *s) {
    if (is_mixed(s))
        launch_fixed_to_rho(s->rho_fixed, s->dm.dv_inv, fixed_unit(s), s->ndof, s->rho_acc, s->rho, s->stream);
    else
        launch_scale(s->rho_acc, s->dm.dv_inv, s->rho, s->ndof, s->stream);
    return PG_OK;
}

// Deposit the current particles into the accumulator (zeroed first).
static int deposit_into_acc(pg_sim *s) {
    if (is_mixed(s)) {
        PG_CUDA(cudaMemsetAsync(s->rho_fixed, 0, sizeof(unsigned long long) * s->ndof, s->stream));
        MixedParams mp;
        fill_mixed(s, mp, 0.0, nullptr, false, 0.0, false, nullptr);
        launch_mixed_pass(s->dm, s->P[s->cur], s->n_slots, mp, false, false, false, true, s->cfg.max_walk_steps,
                          s->rho_fixed, s->state, s->partials, s->n_part, s->ke_dev, s->stream);
    } else {
        PG_CUDA(cudaMemsetAsync(s->rho_acc, 0, sizeof(double) * s->ndof, s->stream));
        if (s->n_slots > 0) launch_deposit(s->dm, s->P[s->cur], s->n_slots, s->d_q, s->rho_acc, s->stream);
    }
    return PG_OK;
}

// Deposit the current particles, then rho = accumulator * dv_inv.
static int deposit_all(pg_sim *s) {
    int rc = deposit_into_acc(s);
    if (rc) return rc;
    s->rho_valid = true;
    return rho_from_acc(s);
}

// CircuitCM::pre_solve + solve + post_solve + correction solve
// (punc/src/poisson.cpp:364-376, punc/src/object_CM.cpp:53-60, 275-376).
static int solve_circuit_internal(pg_sim *s, pg_object *objects, int32_t n_objects, pg_solve_info *info) {
    const int n = s->n_obj;
    std::vector<pg_object *> obj(n, nullptr);
    for (int k = 0; k < n_objects; ++k) {
        const int i = object_index(s, objects[k].bnd_id);
        if (i < 0) return fail(PG_ERR_ARG, "object bnd_id " + std::to_string(objects[k].bnd_id) + " is not an object tag");
        obj[i] = &objects[k];
    }
    for (int i = 0; i < n; ++i)
        if (!obj[i]) return fail(PG_ERR_ARG, "solve_circuit needs every object of the mesh");
    // pre_solve: current sources, potentials to zero
    for (auto &src : s->isrc) {
        const double dQ = src.value * s->circ_dt;
        if (src.node_a != -1) obj[src.node_a]->charge -= dQ;
        if (src.node_b != -1) obj[src.node_b]->charge += dQ;
    }
    std::vector<double> pot(n, 0.0);
    for (int i = 0; i < n; ++i) obj[i]->potential = 0.0;
    const bool superpose = !s->cfg.circuit_resolve && s->lap;
    int rc = superpose ? poisson_solve_internal(s, pot.data(), false, true, s->cfg.pcg_rtol, s->cfg.pcg_atol, info,
                                                s->phi0, &s->phi0_valid)
                       : poisson_solve_internal(s, pot.data(), false, true, s->cfg.pcg_rtol, s->cfg.pcg_atol, info);
    if (rc) return rc;
    // post_solve
    std::vector<double> img;
    rc = image_charges(s, img, superpose ? s->phi0 : s->phi);
    if (rc) return rc;
    std::vector<double> &cv = s->circ_vec;
    for (auto &g : s->groups) {
        double col = 0.0;
        for (int v : g) col += obj[v]->charge;
        cv[n + g[0]] = col;
    }
    for (auto &g : s->groups) {
        double col = 0.0;
        for (int v : g) col += s->inv_cap[g[0] * n + v] * img[v];
        cv[g[0]] = col;
        for (size_t j = 1; j < g.size(); ++j) {
            col = 0.0;
            for (int v : g) col += s->inv_cap[g[j] * n + v] * img[v];
            cv[n + g[j]] = col;
        }
    }
    for (auto &fv : s->fixed_voltage)
        for (size_t j = 0; j < fv.size(); ++j) {
            double col = 0.0;
            for (size_t k = 0; k < fv.size(); ++k) col += s->inv_cap[fv[j] * n + fv[k]] * img[fv[k]];
            cv[n + fv[j]] = col;
        }
    for (int i = 0; i < n; ++i) {
        double p = 0.0, c = 0.0;
        for (int j = 0; j < 2 * n; ++j) p += s->inv_circ[i * 2 * n + j] * cv[j];
        for (int j = 0; j < 2 * n; ++j) c += s->inv_circ[(n + i) * 2 * n + j] * cv[j];
        obj[i]->potential = p;
        obj[i]->charge = c;
        pot[i] = p;
    }
    if (superpose) {
        // the potential is affine in the object potentials: phi = phi0 + sum V_k L_k
        Pots pv{};
        pv.n = n;
        for (int i = 0; i < n; ++i) pv.v[i] = pot[i];
        launch_superpose(s->phi0, s->lap, pv, s->lap_rng, s->ndof, s->phi, s->stream);
        s->phi_valid = true;
        return PG_OK;
    }
    // correction solve with the new potentials
    return poisson_solve_internal(s, pot.data(), false, true, s->cfg.pcg_rtol, s->cfg.pcg_atol, info);
}

static void absorbed_to_objects(pg_sim *s, pg_object *objects, int32_t n_objects, double dt, int64_t *n_absorbed) {
    int64_t tot = 0;
    for (int t = 0; t < kMaxTags; ++t)
        for (int sp = 0; sp < s->n_species; ++sp) tot += s->state_h->absorbed[t][sp];
    if (n_absorbed) *n_absorbed = tot;
    for (int k = 0; k < n_objects; ++k) objects[k].current = 0;
    for (int k = 0; k < n_objects; ++k) {
        const int64_t tag = objects[k].bnd_id;
        if (tag <= 0 || tag >= kMaxTags) continue;
        double cur = 0.0;
        for (int sp = 0; sp < s->n_species; ++sp) cur += (double)s->state_h->absorbed[tag][sp] * s->q[sp];
        objects[k].current = cur;
    }
    for (int k = 0; k < n_objects; ++k) {
        objects[k].charge += objects[k].current;
        objects[k].current /= dt;
    }
}

static int do_sort(pg_sim *s) {
    const int other = 1 - s->cur;
    PG_CUDA(cudaMemsetAsync(s->sort_hist, 0, sizeof(int64_t) * (s->nc + 1), s->stream));
    launch_sort_hist(s->P[s->cur], s->n_slots, s->sort_hist, s->stream);
    launch_scan_i64(s->sort_hist, s->sort_cursor, s->nc + 1, s->scan_tmp, s->stream);
    int64_t total = 0;
    PG_CUDA(cudaMemcpyAsync(&total, s->sort_cursor + s->nc, sizeof(int64_t), cudaMemcpyDeviceToHost, s->stream));
    launch_sort_scatter(s->P[s->cur], s->P[other], s->n_slots, s->sort_cursor, s->stream);
    PG_CUDA(cudaStreamSynchronize(s->stream));
    s->cur = other;
    s->n_slots = total;
    return PG_OK;
}

static int ensure_scan_tmp(pg_sim *s, int64_t n) {
    const int64_t need = scan_tmp_size(n);
    if (need <= s->scan_tmp_n) return PG_OK;
    if (s->scan_tmp) cudaFree(s->scan_tmp);
    s->scan_tmp = nullptr;
    PG_CUDA(cudaMalloc(&s->scan_tmp, sizeof(int64_t) * need));
    s->scan_tmp_n = need;
    return PG_OK;
}

// The FP32 screening boxes of the injected species (the same bits as
// flux_box32 on the device: IEEE conversions and one division).
static void fill_flux32(InjectParams &ip) {
    for (int k = 0; k < ip.n_species; ++k) {
        FluxBox B;
        for (int c = 0; c < 3; ++c) { B.lo[c] = ip.sp[k].domain_lo[c]; B.w[c] = ip.sp[k].domain_w[c]; B.vd[c] = ip.sp[k].vd[c]; }
        B.vth2 = ip.sp[k].vth2;
        B.factor = ip.sp[k].factor;
        ip.sp32[k] = flux_box32(B);
    }
}

// Injection with optional deposit into rho_acc (fused step).
static int inject_internal(pg_sim *s, double dt, uint64_t seed, uint64_t step, bool deposit, int64_t *n_inj) {
    if (!s->flux_ready) return fail(PG_ERR_STATE, "pg_inject: call pg_create_flux first");
    const int total = s->n_inj_species * s->n_ext;
    if (total == 0) { if (n_inj) *n_inj = 0; return PG_OK; }
    InjectParams ip{};
    ip.n_species = s->n_inj_species;
    ip.n_facets = s->n_ext;
    ip.seed = seed;
    ip.step = (uint32_t)step;
    ip.dt = dt;
    int64_t bound = 0;
    for (int k = 0; k < s->n_inj_species; ++k) {
        const pg_species &S = s->inj[k];
        InjectSpecies &I = ip.sp[k];
        I.ndt = S.n * dt;
        const double range = S.vdf_range > 0 ? S.vdf_range : 5.0;
        for (int c = 0; c < 3; ++c) {
            const double lo = S.vd[c] - range * S.vth, hi = S.vd[c] + range * S.vth;
            I.domain_lo[c] = lo;
            I.domain_w[c] = hi - lo;
            I.vd[c] = S.vd[c];
        }
        I.vth2 = S.vth * S.vth;
        I.factor = 1.0 / std::pow(std::sqrt(2. * M_PI * I.vth2), 3);
        I.q = S.q;
        // sum_j (floor(f_j n dt) + 1) <= n dt sum_j f_j + n_facets
        bound += (int64_t)std::ceil(s->flux_sum_h[k] * I.ndt) + s->n_ext;
    }
    int rc = ensure_capacity(s, s->n_slots + bound);
    if (rc) return rc;
    rc = ensure_scan_tmp(s, total + 1);
    if (rc) return rc;
    fill_flux32(ip);
    ip.facets_f = s->d_ext_facets_f;
    // the species slots of the injection table are engine species ids
    InjectParams ipd = ip;
    for (int k = 0; k < ip.n_species; ++k) ipd.sp[k] = ip.sp[k];
    ipd.slot_base = s->n_slots;
    ipd.pid_base = s->next_pid;
    ipd.facet_c1 = s->d_inj_c1;
    ipd.facet_seed = s->d_inj_seed;
    ipd.rho_fixed = s->rho_fixed;
    {
        const double unit = fixed_unit(s);
        for (int k = 0; k < s->n_species; ++k) ipd.q_scaled[k] = (float)(s->q[k] / unit);
    }
    PG_CUDA(cudaMemsetAsync(s->inj_counts, 0, sizeof(int64_t) * (total + 1), s->stream));
    PG_CUDA(cudaMemsetAsync(s->state->injected, 0, sizeof(s->state->injected), s->stream));
    launch_inject_count(s->dm, ipd, s->flux_num, s->inj_counts, s->stream);
    launch_scan_i64(s->inj_counts, s->inj_offsets, total + 1, s->scan_tmp, s->stream);
    launch_inject_generate(s->dm, s->P[s->cur], ipd, s->flux_num, s->pdf_max, s->d_ext_facets, s->inj_offsets,
                           s->cfg.max_walk_steps, deposit ? 1 : 0, s->d_q, s->rho_acc, s->state, bound, s->stream);
    rc = check_state(s);
    if (rc) return rc;
    const int64_t appended = s->state_h->inject_total;
    s->n_slots += appended;
    s->next_pid += appended;
    int64_t kept = 0;
    for (int k = 0; k < kMaxSpecies; ++k) kept += s->state_h->injected[k];
    if (n_inj) *n_inj = kept;
    return PG_OK;
}

static void fill_push(const pg_sim *s, PushParams &pp, double dt, const double *B, bool accel) {
    pp = PushParams{};
    pp.threads = s->tune_threads;
    pp.accel = accel ? 1 : 0;
    pp.has_B = (!accel && B && (B[0] != 0.0 || B[1] != 0.0 || B[2] != 0.0)) ? 1 : 0;
    for (int k = 0; k < s->n_species; ++k) {
        const double q = s->q[k], m = s->m[k];
        pp.coef[k] = accel ? dt * (q / m) : 0.5 * dt * (q / m);
        pp.half_m[k] = 0.5 * m;
        if (pp.has_B) {
            // t = tan((dt q / 2m) B), s = 2t / (1 + |t|^2) (pusher.h:469-479)
            double t[3], t2 = 0.0;
            for (int i = 0; i < 3; ++i) { t[i] = std::tan((dt * q / (2.0 * m)) * B[i]); t2 += t[i] * t[i]; }
            for (int i = 0; i < 3; ++i) { pp.t[k][i] = t[i]; pp.s[k][i] = 2 * t[i] / (1 + t2); }
        }
    }
}

// ---- C ABI -------------------------------------------------------------------

extern "C" {

int pg_create(const pg_mesh *mesh, const pg_config *cfg_in, pg_sim **out) {
    if (!mesh || !out) return fail(PG_ERR_ARG, "pg_create: NULL argument");
    *out = nullptr;
    const HostMesh &h = mesh->h;
    if (h.n_objects >= kMaxTags - 2) return fail(PG_ERR_ARG, "pg_create: too many object tags");
    if (cfg_in && cfg_in->precision == PG_MIXED && cfg_in->particle_capacity > kMaxMixedSlots)
        return fail(PG_ERR_CAPACITY, "pg_create: " + mixed_capacity_message(cfg_in->particle_capacity));
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(PG_ERR_CUDA, "pg_create: no CUDA device");
    pg_sim *s = new pg_sim;
    pg_config cfg = cfg_in ? *cfg_in : pg_config{};
    if (cfg.eps0 == 0) cfg.eps0 = 1.0;
    if (cfg.max_walk_steps <= 0) cfg.max_walk_steps = 100000;
    if (cfg.sort_interval <= 0) cfg.sort_interval = 20;
    if (cfg.pcg_rtol <= 0) cfg.pcg_rtol = 1e-12;
    if (cfg.pcg_atol <= 0) cfg.pcg_atol = 1e-14;
    if (cfg.pcg_max_iter <= 0) cfg.pcg_max_iter = 1000;
    s->cfg = cfg;
    auto bail = [&](int rc) { pg_destroy(s); return rc; };
    cudaGetDevice(&s->device);
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(PG_ERR_CUDA, "cudaStreamCreate failed"));
    s->nc = (int32_t)h.nc;
    s->ndof = (int32_t)h.ndof;
    s->n_obj = h.n_objects;

    // mesh tables
    std::vector<int32_t> nbr32(4 * h.nc), dof32(4 * h.nc);
    for (int64_t k = 0; k < 4 * h.nc; ++k) { nbr32[k] = (int32_t)h.nbr[k]; dof32[k] = (int32_t)h.cell_dofs[k]; }
    double *d_planes, *d_bary, *d_E, *d_dvinv;
    int32_t *d_nbr, *d_dofs;
    int rc;
    if ((rc = upload(s, &d_planes, h.planes)) || (rc = upload(s, &d_bary, h.bary)) || (rc = upload(s, &d_nbr, nbr32)) ||
        (rc = upload(s, &d_dofs, dof32)) || (rc = upload(s, &d_dvinv, h.dv_inv)) || (rc = dalloc(s, &d_E, 4 * h.nc)))
        return bail(rc);
    cudaMemset(d_E, 0, sizeof(double) * 4 * h.nc);
    if (cfg.precision == PG_MIXED) {
        float4 *cf;
        float *ef;
        if ((rc = dalloc(s, &cf, 4 * h.nc)) || (rc = dalloc(s, &ef, 4 * h.nc)) || (rc = dalloc(s, &s->rho_fixed, h.ndof)))
            return bail(rc);
        cudaMemset(ef, 0, sizeof(float) * 4 * h.nc);
        cudaMemset(s->rho_fixed, 0, sizeof(unsigned long long) * h.ndof);
        launch_float_tables(d_bary, reinterpret_cast<const int4 *>(d_nbr), (int32_t)h.nc, cf, s->stream);
        s->dm.cell_f = cf;
        s->dm.E_f = ef;
    } else if (cfg.precision != PG_FP64) {
        return bail(fail(PG_ERR_ARG, "pg_create: unknown precision"));
    }
    s->dm.nc = s->nc;
    s->dm.ndof = s->ndof;
    s->dm.planes = d_planes;
    s->dm.bary = d_bary;
    s->dm.nbr = reinterpret_cast<const int4 *>(d_nbr);
    s->dm.dofs = reinterpret_cast<const int4 *>(d_dofs);
    s->dm.E = d_E;
    s->dm.dv_inv = d_dvinv;
    for (int j = 0; j < 3; ++j) { s->dm.lo[j] = h.bbox_lo[j]; s->dm.bin_h[j] = h.bin_h[j]; s->dm.nbin[j] = h.nbin[j]; }
    int64_t *d_binptr;
    int32_t *d_bincells;
    if ((rc = upload(s, &d_binptr, h.bin_ptr)) || (rc = upload(s, &d_bincells, h.bin_cells))) return bail(rc);
    s->dm.bin_ptr = d_binptr;
    s->dm.bin_cells = d_bincells;

    // fields
    if ((rc = dalloc(s, &s->rho_acc, h.ndof)) || (rc = dalloc(s, &s->rho, h.ndof)) || (rc = dalloc(s, &s->phi, h.ndof)) ||
        (rc = dalloc(s, &s->b, h.ndof)))
        return bail(rc);
    cudaMemset(s->rho_acc, 0, sizeof(double) * h.ndof);
    cudaMemset(s->rho, 0, sizeof(double) * h.ndof);
    cudaMemset(s->phi, 0, sizeof(double) * h.ndof);

    // Poisson: symmetric elimination of Dirichlet rows and columns.
    {
        const int64_t nd = h.ndof;
        std::vector<int32_t> kind(nd);
        s->has_dirichlet = false;
        for (int64_t i = 0; i < nd; ++i) {
            kind[i] = cfg.periodic ? -1 : (int32_t)h.bc_kind[i];
            if (kind[i] >= 0) s->has_dirichlet = true;
        }
        std::vector<double> gval(nd, 0.0);
        if (!cfg.periodic) {
            for (int64_t c = 0; c < h.nc; ++c)
                for (int i = 0; i < 4; ++i) {
                    const int64_t v = h.cell_vertices[4 * c + i], d = h.cell_dofs[4 * c + i];
                    double val = 0.0;
                    for (int j = 0; j < 3; ++j) val += h.coords[3 * v + j] * cfg.ext_E[j];
                    gval[d] = val;
                }
        }
        std::vector<int32_t> arow(nd + 1, 0), acol, mrow(nd + 1), mcol(h.col.size());
        std::vector<double> aval, dinv(nd, 1.0), wext(nd, 0.0), wobj((size_t)std::max(1, s->n_obj) * nd, 0.0);
        acol.reserve(h.col.size());
        aval.reserve(h.col.size());
        for (int64_t i = 0; i < nd; ++i) {
            if (kind[i] >= 0) {
                acol.push_back((int32_t)i);
                aval.push_back(1.0);
            } else {
                for (int64_t k = h.rowptr[i]; k < h.rowptr[i + 1]; ++k) {
                    const int64_t j = h.col[k];
                    if (kind[j] < 0) {
                        if (h.K[k] == 0.0 && j != i) continue;   // exact zeros of K add nothing
                        acol.push_back((int32_t)j);
                        aval.push_back(h.K[k]);
                        if (j == i) dinv[i] = 1.0 / h.K[k];
                    } else if (kind[j] == 0) {
                        wext[i] += h.K[k] * gval[j];
                    } else {
                        wobj[(size_t)(kind[j] - 1) * nd + i] += h.K[k];
                    }
                }
            }
            arow[i + 1] = (int32_t)acol.size();
        }
        for (int64_t i = 0; i <= nd; ++i) mrow[i] = (int32_t)h.rowptr[i];
        for (size_t k = 0; k < h.col.size(); ++k) mcol[k] = (int32_t)h.col[k];
        {
            // M in SELL-32 (rows' entries in CSR order; padding: value 0, own column)
            const int64_t msl = (nd + 31) / 32;
            std::vector<int64_t> mp(msl + 1, 0);
            std::vector<int32_t> mw(msl, 0);
            for (int64_t sl = 0; sl < msl; ++sl) {
                int32_t w = 0;
                for (int64_t r = 32 * sl; r < std::min<int64_t>(nd, 32 * sl + 32); ++r)
                    w = std::max<int32_t>(w, (int32_t)(h.rowptr[r + 1] - h.rowptr[r]));
                mw[sl] = w;
                mp[sl + 1] = mp[sl] + 32 * (int64_t)w;
            }
            std::vector<int32_t> mc(std::max<int64_t>(1, mp[msl]), 0);
            std::vector<double> mv(std::max<int64_t>(1, mp[msl]), 0.0);
            for (int64_t sl = 0; sl < msl; ++sl)
                for (int lane = 0; lane < 32; ++lane) {
                    const int64_t r = 32 * sl + lane;
                    const int64_t len = r < nd ? h.rowptr[r + 1] - h.rowptr[r] : 0;
                    for (int32_t k = 0; k < mw[sl]; ++k) {
                        const int64_t o = mp[sl] + 32 * (int64_t)k + lane;
                        if (k < len) { mc[o] = (int32_t)h.col[h.rowptr[r] + k]; mv[o] = h.M[h.rowptr[r] + k]; }
                        else mc[o] = (int32_t)std::min<int64_t>(r, nd - 1);
                    }
                }
            if ((rc = upload(s, &s->Ms_ptr, mp)) || (rc = upload(s, &s->Ms_width, mw)) ||
                (rc = upload(s, &s->Ms_col, mc)) || (rc = upload(s, &s->Ms_val, mv)))
                return bail(rc);
        }
        // SELL-32: slice s holds rows 32s..32s+31 column-major, padded with (row, 0.0)
        const int64_t nsl = (nd + 31) / 32;
        std::vector<int64_t> sptr(nsl + 1, 0);
        std::vector<int32_t> swidth(nsl, 0);
        for (int64_t sl = 0; sl < nsl; ++sl) {
            int32_t w = 0;
            for (int64_t r = 32 * sl; r < std::min(nd, 32 * sl + 32); ++r) w = std::max(w, arow[r + 1] - arow[r]);
            swidth[sl] = w;
            sptr[sl + 1] = sptr[sl] + 32 * (int64_t)w;
        }
        std::vector<int32_t> scol(sptr[nsl]);
        std::vector<double> sval(sptr[nsl], 0.0);
        for (int64_t sl = 0; sl < nsl; ++sl)
            for (int lane = 0; lane < 32; ++lane) {
                const int64_t r = 32 * sl + lane;
                const int32_t len = r < nd ? arow[r + 1] - arow[r] : 0;
                for (int32_t k = 0; k < swidth[sl]; ++k) {
                    const int64_t o = sptr[sl] + 32 * (int64_t)k + lane;
                    if (k < len) { scol[o] = acol[arow[r] + k]; sval[o] = aval[arow[r] + k]; }
                    else { scol[o] = (int32_t)std::min<int64_t>(r, nd - 1); sval[o] = 0.0; }
                }
            }
        if ((rc = upload(s, &s->A_sptr, sptr)) || (rc = upload(s, &s->A_swidth, swidth)) ||
            (rc = upload(s, &s->A_col, scol)) || (rc = upload(s, &s->A_val, sval)) || (rc = dalloc(s, &s->phi0, nd)) ||
            (rc = upload(s, &s->A_dinv, dinv)) || (rc = upload(s, &s->M_row, mrow)) || (rc = upload(s, &s->M_col, mcol)) ||
            (rc = upload(s, &s->M_val, h.M)) || (rc = upload(s, &s->bc_kind, kind)) || (rc = upload(s, &s->bc_value, gval)) ||
            (rc = upload(s, &s->w_ext, wext)) || (rc = upload(s, &s->w_obj, wobj)))
            return bail(rc);
        const int nb = std::max(pcg_grid_blocks(), pcg_amg_grid_blocks());
        if ((rc = dalloc(s, &s->r, nd)) || (rc = dalloc(s, &s->z, nd)) || (rc = dalloc(s, &s->p0, nd)) ||
            (rc = dalloc(s, &s->p1, nd)) || (rc = dalloc(s, &s->Ap, nd)) || (rc = dalloc(s, &s->pcg_part, 4 * nb)) ||
            (rc = dalloc(s, &s->pcg_out_i, 2)) || (rc = dalloc(s, &s->pcg_out_d, 2)) ||
            (rc = dalloc(s, &s->obj_pot, std::max(1, s->n_obj))) || (rc = dalloc(s, &s->image, std::max(1, s->n_obj))))
            return bail(rc);
        if (cfg.pcg_precond != 0 && cfg.pcg_precond != 1) return bail(fail(PG_ERR_ARG, "pg_create: unknown pcg_precond"));
        const bool amg = cfg.pcg_precond == 0;
        const int mode = amg ? 2 : (cfg.pcg_precision == 0 ? (cfg.precision == PG_MIXED ? 2 : 1) : cfg.pcg_precision);
        s->a_nnz = (int64_t)acol.size();
        s->a_sell = sptr[nsl];
        if (mode == 2) {
            std::vector<float> v32(sval.begin(), sval.end()), d32(dinv.begin(), dinv.end());
            if ((rc = upload(s, &s->A_val32, v32)) || (rc = upload(s, &s->A_dinv32, d32)) ||
                (rc = dalloc(s, &s->r32, nd)) || (rc = dalloc(s, &s->z32, nd)) || (rc = dalloc(s, &s->p32, nd)) ||
                (rc = dalloc(s, &s->Ap32, nd)))
                return bail(rc);
        } else if (mode != 1) {
            return bail(fail(PG_ERR_ARG, "pg_create: unknown pcg_precision"));
        }
        if (amg && (rc = setup_amg(s, arow, acol, aval))) return bail(rc);
    }

    // ESolver: dof -> cell adjacency in ascending cell order, volumes, D^-1 of
    // the mass matrix, work arrays, the packed vertex field
    {
        const int64_t nd = h.ndof, ncell = h.nc;
        std::vector<int64_t> aptr(nd + 1, 0);
        for (int64_t k = 0; k < 4 * ncell; ++k) aptr[h.cell_dofs[k] + 1]++;
        for (int64_t d = 0; d < nd; ++d) aptr[d + 1] += aptr[d];
        std::vector<int32_t> acell(4 * ncell);
        std::vector<int64_t> cur(aptr.begin(), aptr.end() - 1);
        for (int64_t c = 0; c < ncell; ++c)
            for (int i = 0; i < 4; ++i) acell[cur[h.cell_dofs[4 * c + i]]++] = (int32_t)c;
        std::vector<double> mdinv(nd, 1.0);
        for (int64_t i = 0; i < nd; ++i)
            for (int64_t k = h.rowptr[i]; k < h.rowptr[i + 1]; ++k)
                if (h.col[k] == i && h.M[k] != 0.0) mdinv[i] = 1.0 / h.M[k];
        if ((rc = upload(s, &s->es_adj_ptr, aptr)) || (rc = upload(s, &s->es_adj_cell, acell)) ||
            (rc = upload(s, &s->es_vol, h.volume)) || (rc = upload(s, &s->M_dinv, mdinv)) ||
            (rc = dalloc(s, &s->es_part, 12 * std::max(1, esolve_grid_blocks()))) || (rc = dalloc(s, &s->es_out_i, 2)) ||
            (rc = dalloc(s, &s->es_out_d, 6)) || (rc = dalloc(s, &s->Ev, 4 * nd)))
            return bail(rc);
        cudaMemset(s->Ev, 0, sizeof(double) * 4 * nd);
        if (cfg.precision == PG_MIXED) {
            std::vector<float> m32(h.M.begin(), h.M.end()), d32(mdinv.begin(), mdinv.end());
            if ((rc = upload(s, &s->M_val32, m32)) || (rc = upload(s, &s->M_dinv32, d32)) ||
                (rc = dalloc(s, &s->es_buf32, 18 * nd)) || (rc = dalloc(s, &s->Evf, 4 * nd)))
                return bail(rc);
            cudaMemset(s->es_buf32, 0, sizeof(float) * 18 * nd);
            cudaMemset(s->Evf, 0, sizeof(float) * 4 * nd);
        } else {
            if ((rc = dalloc(s, &s->es_buf, 18 * nd))) return bail(rc);
            cudaMemset(s->es_buf, 0, sizeof(double) * 18 * nd);
        }
        s->dm.Ev = s->Ev;
        s->dm.Evf = s->Evf;
    }

    // boundary facets
    s->ext_facets_h = h.ext_facets;
    s->obj_facets_h = h.obj_facets;
    s->n_ext = (int32_t)(h.ext_facets.size() / 14);
    s->n_ofac = (int32_t)(h.obj_facets.size() / 7);
    if ((rc = upload(s, &s->d_ext_facets, h.ext_facets)) || (rc = upload(s, &s->d_ofacets, h.obj_facets))) return bail(rc);
    if (cfg.precision == PG_MIXED && s->n_ext > 0) {
        std::vector<float4> ff(4 * (size_t)s->n_ext);
        for (int64_t j = 0; j < s->n_ext; ++j) {
            const double *F = &h.ext_facets[14 * (size_t)j];
            float v[12];
            for (int k = 0; k < 12; ++k) v[k] = (float)F[1 + k];
            int cellj = (int)F[13];
            ff[4 * j] = make_float4(v[0], v[1], v[2], v[3]);
            ff[4 * j + 1] = make_float4(v[4], v[5], v[6], v[7]);
            ff[4 * j + 2] = make_float4(v[8], v[9], v[10], v[11]);
            float cf;
            std::memcpy(&cf, &cellj, sizeof(cf));
            ff[4 * j + 3] = make_float4(cf, 0.0f, 0.0f, 0.0f);
        }
        if ((rc = upload(s, &s->d_ext_facets_f, ff))) return bail(rc);
    }

    // state, reductions, sort scratch
    if ((rc = dalloc(s, &s->state, 1))) return bail(rc);
    cudaMemset(s->state, 0, sizeof(DevState));
    if (cudaMallocHost(&s->state_h, sizeof(DevState)) != cudaSuccess) return bail(fail(PG_ERR_CUDA, "cudaMallocHost failed"));
    std::memset(s->state_h, 0, sizeof(DevState));
    s->n_part = sm_count() * 8;
    s->part_cap = sm_count() * 32;
    if ((rc = dalloc(s, &s->partials, s->part_cap)) || (rc = dalloc(s, &s->ke_dev, 1)) || (rc = dalloc(s, &s->d_q, kMaxSpecies)))
        return bail(rc);
    cudaMemset(s->d_q, 0, sizeof(double) * kMaxSpecies);
    if ((rc = dalloc(s, &s->sort_hist, h.nc + 1)) || (rc = dalloc(s, &s->sort_cursor, h.nc + 1))) return bail(rc);
    if ((rc = ensure_scan_tmp(s, h.nc + 1))) return bail(rc);
    if (cfg.particle_capacity > 0) {
        if ((rc = alloc_particles(s, s->P[0], cfg.particle_capacity)) || (rc = alloc_particles(s, s->P[1], cfg.particle_capacity)))
            return bail(rc);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return bail(fail(PG_ERR_CUDA, "pg_create: device error during upload"));
    *out = s;
    return PG_OK;
}

int pg_destroy(pg_sim *s) {
    if (!s) return PG_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (auto &g : s->graph_exec)
        if (g) cudaGraphExecDestroy(g);
    for (void *p : s->adj.mem) cudaFree(p);
    for (void *p : s->amg_mem) cudaFree(p);
    for (void *p : s->allocs) cudaFree(p);
    free_particles(s->P[0]);
    free_particles(s->P[1]);
    if (s->flux_num) cudaFree(s->flux_num);
    if (s->pdf_max) cudaFree(s->pdf_max);
    if (s->inj_counts) cudaFree(s->inj_counts);
    if (s->inj_offsets) cudaFree(s->inj_offsets);
    if (s->scan_tmp) cudaFree(s->scan_tmp);
    if (s->state_h) cudaFreeHost(s->state_h);
    for (auto &e : s->ev_pending) { cudaEventDestroy(e.second.first); cudaEventDestroy(e.second.second); }
    for (auto &e : s->user_ev)
        if (e) cudaEventDestroy(e);
    if (s->copy_stream) {
        cudaStreamSynchronize(s->copy_stream);
        cudaStreamDestroy(s->copy_stream);
    }
    if (s->phi_ready) cudaEventDestroy(s->phi_ready);
    if (s->phi_copied) cudaEventDestroy(s->phi_copied);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return PG_OK;
}

int pg_status_detail(pg_sim *s, int32_t *code, int64_t *index) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    PG_CUDA(cudaMemcpyAsync(s->state_h, s->state, sizeof(DevState), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    if (code) *code = s->state_h->err_code;
    if (index) *index = s->state_h->err_index;
    return PG_OK;
}

static int add_particles_internal(pg_sim *s, const double *xs, const double *vs, int64_t n, double q, double m,
                                  int32_t cell_lo, int32_t cell_hi, int64_t *n_added);

int pg_add_particles(pg_sim *s, const double *xs, const double *vs, int64_t n, double q, double m, int64_t *n_added) {
    return add_particles_internal(s, xs, vs, n, q, m, 0, 0x7fffffff, n_added);
}

int pg_add_particles_range(pg_sim *s, const double *xs, const double *vs, int64_t n, double q, double m,
                           int32_t cell_lo, int32_t cell_hi, int64_t *n_added) {
    if (s && (cell_lo < 0 || cell_hi <= cell_lo)) return fail(PG_ERR_ARG, "pg_add_particles_range: empty cell range");
    return add_particles_internal(s, xs, vs, n, q, m, cell_lo, cell_hi, n_added);
}

int pg_set_injection_streams(pg_sim *s, const uint32_t *facet_stream, const uint64_t *facet_seed) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    int rc;
    if (facet_stream) {
        std::vector<uint32_t> v(facet_stream, facet_stream + s->n_ext);
        if (!s->d_inj_c1 && (rc = dalloc(s, &s->d_inj_c1, std::max(1, s->n_ext)))) return rc;
        PG_CUDA(cudaMemcpy(s->d_inj_c1, v.data(), sizeof(uint32_t) * v.size(), cudaMemcpyHostToDevice));
    }
    if (facet_seed) {
        std::vector<uint64_t> v(facet_seed, facet_seed + s->n_ext);
        if (!s->d_inj_seed && (rc = dalloc(s, &s->d_inj_seed, std::max(1, s->n_ext)))) return rc;
        PG_CUDA(cudaMemcpy(s->d_inj_seed, v.data(), sizeof(uint64_t) * v.size(), cudaMemcpyHostToDevice));
    }
    return PG_OK;
}

static int add_particles_internal(pg_sim *s, const double *xs, const double *vs, int64_t n, double q, double m,
                                  int32_t cell_lo, int32_t cell_hi, int64_t *n_added) {
    if (!s || (n > 0 && (!xs || !vs)) || n < 0) return fail(PG_ERR_ARG, "pg_add_particles: bad arguments");
    if (n_added) *n_added = 0;
    if (n == 0) return PG_OK;
    const int sp = species_id(s, q, m);
    if (sp < 0) return fail(PG_ERR_ARG, "pg_add_particles: more than 8 species");
    // the mixed form stores FP32 positions: locate the rounded points
    std::vector<double> rounded;
    const double *pos = xs;
    if (is_mixed(s)) {
        rounded.resize(3 * n);
        for (int64_t k = 0; k < 3 * n; ++k) rounded[k] = (double)(float)xs[k];
        pos = rounded.data();
    }
    double *d_xyz = nullptr;
    int32_t *d_cells = nullptr;
    PG_CUDA(cudaMalloc(&d_xyz, sizeof(double) * 3 * n));
    PG_CUDA(cudaMalloc(&d_cells, sizeof(int32_t) * n));
    std::vector<int32_t> cells(n);
    cudaMemcpyAsync(d_xyz, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s->stream);
    DevMesh dm = s->dm;
    dm.loc_lo = cell_lo;
    dm.loc_hi = cell_hi;
    launch_locate(dm, d_xyz, n, d_cells, s->stream);
    cudaMemcpyAsync(cells.data(), d_cells, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    cudaFree(d_xyz);
    cudaFree(d_cells);
    if (e != cudaSuccess) return fail(PG_ERR_CUDA, std::string("pg_add_particles: ") + cudaGetErrorString(e));
    std::vector<double> hx, hy, hz, hvx, hvy, hvz;
    std::vector<int32_t> hc;
    std::vector<uint8_t> hs;
    std::vector<int64_t> hp;
    for (int64_t i = 0; i < n; ++i) {
        if (cells[i] < 0) continue;
        hx.push_back(xs[3 * i]); hy.push_back(xs[3 * i + 1]); hz.push_back(xs[3 * i + 2]);
        hvx.push_back(vs[3 * i]); hvy.push_back(vs[3 * i + 1]); hvz.push_back(vs[3 * i + 2]);
        hc.push_back(cells[i]);
        hs.push_back((uint8_t)sp);
        hp.push_back(s->next_pid + i);
    }
    const int64_t k = (int64_t)hx.size();
    int rc = ensure_capacity(s, s->n_slots + k);
    if (rc) return rc;
    const DevParticles &P = s->P[s->cur];
    const int64_t o = s->n_slots;
    if (is_mixed(s)) {
        auto up = [&](float *dst, const std::vector<double> &src) {
            std::vector<float> f(src.begin(), src.end());
            return cudaMemcpy(dst + o, f.data(), 4 * k, cudaMemcpyHostToDevice);
        };
        PG_CUDA(up(P.xf, hx)); PG_CUDA(up(P.yf, hy)); PG_CUDA(up(P.zf, hz));
        PG_CUDA(up(P.vxf, hvx)); PG_CUDA(up(P.vyf, hvy)); PG_CUDA(up(P.vzf, hvz));
    } else {
        PG_CUDA(cudaMemcpy(P.x + o, hx.data(), 8 * k, cudaMemcpyHostToDevice));
        PG_CUDA(cudaMemcpy(P.y + o, hy.data(), 8 * k, cudaMemcpyHostToDevice));
        PG_CUDA(cudaMemcpy(P.z + o, hz.data(), 8 * k, cudaMemcpyHostToDevice));
        PG_CUDA(cudaMemcpy(P.vx + o, hvx.data(), 8 * k, cudaMemcpyHostToDevice));
        PG_CUDA(cudaMemcpy(P.vy + o, hvy.data(), 8 * k, cudaMemcpyHostToDevice));
        PG_CUDA(cudaMemcpy(P.vz + o, hvz.data(), 8 * k, cudaMemcpyHostToDevice));
    }
    PG_CUDA(cudaMemcpy(P.cell + o, hc.data(), 4 * k, cudaMemcpyHostToDevice));
    PG_CUDA(cudaMemcpy(P.sp + o, hs.data(), k, cudaMemcpyHostToDevice));
    PG_CUDA(cudaMemcpy(P.pid + o, hp.data(), 8 * k, cudaMemcpyHostToDevice));
    s->n_slots += k;
    s->next_pid += n;
    // live count
    PG_CUDA(cudaMemcpy(s->state_h, s->state, sizeof(DevState), cudaMemcpyDeviceToHost));
    s->state_h->live[sp] += k;
    PG_CUDA(cudaMemcpy(s->state, s->state_h, sizeof(DevState), cudaMemcpyHostToDevice));
    s->rho_valid = false;
    if (n_added) *n_added = k;
    // loaded points come in any order: sort by cell so cell tables are read once per warp
    if (k > 0) return do_sort(s);
    return PG_OK;
}

int pg_num_particles(pg_sim *s, int64_t *total, int64_t *neg, int64_t *pos) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    int rc = check_state(s);
    if (rc) return rc;
    int64_t t = 0, ng = 0, ps = 0;
    for (int k = 0; k < s->n_species; ++k) {
        t += s->state_h->live[k];
        if (s->q[k] < 0) ng += s->state_h->live[k];
        if (s->q[k] > 0) ps += s->state_h->live[k];
    }
    if (total) *total = t;
    if (neg) *neg = ng;
    if (pos) *pos = ps;
    return PG_OK;
}

int pg_get_particles(pg_sim *s, int64_t capacity, double *x, double *v, double *q, double *m, int64_t *cell,
                     int64_t *pid, int64_t *n_out) {
    if (!s || !n_out) return fail(PG_ERR_ARG, "pg_get_particles: NULL argument");
    const int64_t n = s->n_slots;
    const DevParticles &P = s->P[s->cur];
    const bool want = x || v || q || m || cell || pid;
    std::vector<int32_t> hc(n);
    PG_CUDA(cudaStreamSynchronize(s->stream));
    if (n > 0) PG_CUDA(cudaMemcpy(hc.data(), P.cell, 4 * n, cudaMemcpyDeviceToHost));
    if (!want) {
        // count only
        int64_t k = 0;
        for (int64_t i = 0; i < n; ++i) k += hc[i] >= 0;
        *n_out = k;
        return PG_OK;
    }
    // only the requested arrays cross to the host; ids always (sort key)
    std::vector<double> hx(x ? n : 0), hy(x ? n : 0), hz(x ? n : 0), hvx(v ? n : 0), hvy(v ? n : 0), hvz(v ? n : 0);
    std::vector<uint8_t> hs((q || m) ? n : 0);
    std::vector<int64_t> hp(n);
    if (n > 0 && is_mixed(s)) {
        std::vector<float> f(n);
        auto dn = [&](std::vector<double> &dst, const float *src) {
            cudaError_t e = cudaMemcpy(f.data(), src, 4 * n, cudaMemcpyDeviceToHost);
            for (int64_t i = 0; i < n; ++i) dst[i] = f[i];
            return e;
        };
        if (x) { PG_CUDA(dn(hx, P.xf)); PG_CUDA(dn(hy, P.yf)); PG_CUDA(dn(hz, P.zf)); }
        if (v) { PG_CUDA(dn(hvx, P.vxf)); PG_CUDA(dn(hvy, P.vyf)); PG_CUDA(dn(hvz, P.vzf)); }
    } else if (n > 0) {
        if (x) {
            PG_CUDA(cudaMemcpy(hx.data(), P.x, 8 * n, cudaMemcpyDeviceToHost));
            PG_CUDA(cudaMemcpy(hy.data(), P.y, 8 * n, cudaMemcpyDeviceToHost));
            PG_CUDA(cudaMemcpy(hz.data(), P.z, 8 * n, cudaMemcpyDeviceToHost));
        }
        if (v) {
            PG_CUDA(cudaMemcpy(hvx.data(), P.vx, 8 * n, cudaMemcpyDeviceToHost));
            PG_CUDA(cudaMemcpy(hvy.data(), P.vy, 8 * n, cudaMemcpyDeviceToHost));
            PG_CUDA(cudaMemcpy(hvz.data(), P.vz, 8 * n, cudaMemcpyDeviceToHost));
        }
    }
    if (n > 0) {
        if (q || m) PG_CUDA(cudaMemcpy(hs.data(), P.sp, n, cudaMemcpyDeviceToHost));
        PG_CUDA(cudaMemcpy(hp.data(), P.pid, 8 * n, cudaMemcpyDeviceToHost));
    }
    std::vector<int64_t> idx;
    idx.reserve(n);
    for (int64_t i = 0; i < n; ++i)
        if (hc[i] >= 0) idx.push_back(i);
    const int64_t k = (int64_t)idx.size();
    *n_out = k;
    if (k > capacity) return fail(PG_ERR_ARG, "pg_get_particles: capacity too small");
    std::sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return hc[a] != hc[b] ? hc[a] < hc[b] : hp[a] < hp[b]; });
    for (int64_t t = 0; t < k; ++t) {
        const int64_t i = idx[t];
        if (x) { x[3 * t] = hx[i]; x[3 * t + 1] = hy[i]; x[3 * t + 2] = hz[i]; }
        if (v) { v[3 * t] = hvx[i]; v[3 * t + 1] = hvy[i]; v[3 * t + 2] = hvz[i]; }
        if (q) q[t] = s->q[hs[i]];
        if (m) m[t] = s->m[hs[i]];
        if (cell) cell[t] = hc[i];
        if (pid) pid[t] = hp[i];
    }
    return PG_OK;
}

int pg_locate(pg_sim *s, const double *xs, int64_t n, int64_t *cells) {
    if (!s || (n > 0 && (!xs || !cells)) || n < 0) return fail(PG_ERR_ARG, "pg_locate: bad arguments");
    if (n == 0) return PG_OK;
    double *d_xyz = nullptr;
    int32_t *d_cells = nullptr;
    PG_CUDA(cudaMalloc(&d_xyz, sizeof(double) * 3 * n));
    PG_CUDA(cudaMalloc(&d_cells, sizeof(int32_t) * n));
    std::vector<int32_t> c(n);
    cudaMemcpyAsync(d_xyz, xs, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s->stream);
    launch_locate(s->dm, d_xyz, n, d_cells, s->stream);
    cudaMemcpyAsync(c.data(), d_cells, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    cudaFree(d_xyz);
    cudaFree(d_cells);
    if (e != cudaSuccess) return fail(PG_ERR_CUDA, std::string("pg_locate: ") + cudaGetErrorString(e));
    for (int64_t i = 0; i < n; ++i) cells[i] = c[i];
    return PG_OK;
}

int pg_relocate(pg_sim *s, const double *xs, const int64_t *cells, int64_t n, int32_t mode, int64_t *cells_out,
                int32_t *crossings) {
    if (!s || (n > 0 && (!xs || !cells || !cells_out)) || n < 0 || (mode != 0 && mode != 1))
        return fail(PG_ERR_ARG, "pg_relocate: bad arguments");
    if (n == 0) return PG_OK;
    std::vector<int32_t> start(n);
    for (int64_t i = 0; i < n; ++i) {
        if (cells[i] < 0 || cells[i] >= s->nc) return fail(PG_ERR_ARG, "pg_relocate: start cell out of range");
        start[i] = (int32_t)cells[i];
    }
    double *d_xyz = nullptr;
    int32_t *d_io = nullptr;
    PG_CUDA(cudaMalloc(&d_xyz, sizeof(double) * 3 * n));
    if (cudaMalloc(&d_io, sizeof(int32_t) * 3 * n) != cudaSuccess) {
        cudaFree(d_xyz);
        return fail(PG_ERR_CUDA, "pg_relocate: cudaMalloc failed");
    }
    std::vector<int32_t> out(2 * n);
    cudaMemcpyAsync(d_xyz, xs, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(d_io, start.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s->stream);
    launch_relocate(s->dm, d_xyz, d_io, n, mode, s->cfg.max_walk_steps, d_io + n, d_io + 2 * n, s->stream);
    cudaMemcpyAsync(out.data(), d_io + n, sizeof(int32_t) * 2 * n, cudaMemcpyDeviceToHost, s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    cudaFree(d_xyz);
    cudaFree(d_io);
    if (e != cudaSuccess) return fail(PG_ERR_CUDA, std::string("pg_relocate: ") + cudaGetErrorString(e));
    int64_t bad = -1;
    for (int64_t i = 0; i < n; ++i) {
        if (out[i] == kWalkFail && bad < 0) bad = i;
        cells_out[i] = out[i];
        if (crossings) crossings[i] = out[n + i];
    }
    if (bad >= 0) return fail(PG_ERR_WALK_LIMIT, "pg_relocate: walk step limit reached at point " + std::to_string(bad));
    return PG_OK;
}

// ESolver::solve (punc/src/efield.cpp:70-75): E = L2 projection of -grad(phi)
// onto CG1 vector fields, plus the uniform E0, into the packed vertex field.
// FP64 form: FP64 CG to the reference's tolerances (rel 1e-12, abs 1e-14);
// mixed form: FP32 CG to rel 1e-6 (the FP32 push reads the field in FP32).
static int esolver_internal(pg_sim *s, const double E0[3], pg_solve_info *info) {
    const double zero[3] = {0, 0, 0};
    launch_efield(s->dm, s->phi, zero, s->stream);
    EsolveArgs e{};
    e.n = s->ndof;
    e.fp32 = is_mixed(s) ? 1 : 0;
    e.adj_ptr = s->es_adj_ptr; e.adj_cell = s->es_adj_cell; e.vol = s->es_vol; e.E_cell = s->dm.E;
    e.row = s->M_row; e.col = s->M_col; e.val = s->M_val; e.dinv = s->M_dinv;
    e.val32 = s->M_val32; e.dinv32 = s->M_dinv32;
    const size_t n3 = 3 * (size_t)s->ndof;
    if (e.fp32) {
        float *b = s->es_buf32;
        e.b32 = b; e.x32 = b + n3; e.r32 = b + 2 * n3; e.z32 = b + 3 * n3; e.p32 = b + 4 * n3; e.Ap32 = b + 5 * n3;
        e.rtol = 1e-6;
    } else {
        double *b = s->es_buf;
        e.b = b; e.x = b + n3; e.r = b + 2 * n3; e.z = b + 3 * n3; e.p = b + 4 * n3; e.Ap = b + 5 * n3;
        e.rtol = 1e-12;
    }
    e.atol = 1e-14;
    e.max_iter = 1000;
    e.partials = s->es_part;
    e.out_iter = s->es_out_i; e.out_status = s->es_out_i + 1;
    e.out_rr = s->es_out_d; e.out_bb = s->es_out_d + 3;
    for (int j = 0; j < 3; ++j) e.E0[j] = E0 ? E0[j] : 0.0;
    e.ev = s->Ev;
    e.evf = s->Evf;
    int err;
    {
        StageScope t(s, "efield");
        err = launch_esolve(e, s->stream);
    }
    if (err) return fail(PG_ERR_CUDA, std::string("ESolver launch: ") + cudaGetErrorString((cudaError_t)err));
    int32_t oi[2];
    double od[6];
    PG_CUDA(cudaMemcpyAsync(oi, s->es_out_i, sizeof(oi), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaMemcpyAsync(od, s->es_out_d, sizeof(od), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    if (info) {
        info->iterations = oi[0];
        info->solves = 1;
        info->residual = std::sqrt(od[0] + od[1] + od[2]);
        info->rhs_norm = std::sqrt(od[3] + od[4] + od[5]);
    }
    if (oi[1] != 0) return fail(PG_ERR_NOT_CONVERGED, "ESolver: CG on the mass matrix did not converge");
    return PG_OK;
}

int pg_esolver_solve(pg_sim *s, double *E, pg_solve_info *info) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    int rc = esolver_internal(s, nullptr, info);
    if (rc) return rc;
    return E ? pg_get_efield_cg1(s, E) : PG_OK;
}

int pg_set_efield_cg1(pg_sim *s, const double *E) {
    if (!s || !E) return fail(PG_ERR_ARG, "pg_set_efield_cg1: NULL argument");
    const size_t n = (size_t)s->ndof;
    std::vector<double> x3(3 * n);
    for (size_t d = 0; d < n; ++d)
        for (int j = 0; j < 3; ++j) x3[j * n + d] = E[3 * d + j];
    double *tmp = nullptr;
    PG_CUDA(cudaMalloc(&tmp, sizeof(double) * x3.size()));
    cudaError_t e = cudaMemcpy(tmp, x3.data(), sizeof(double) * x3.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const double zero[3] = {0, 0, 0};
        launch_pack_ev64(s->ndof, tmp, zero, s->Ev, s->Evf, s->stream);
        e = cudaStreamSynchronize(s->stream);
    }
    cudaFree(tmp);
    if (e != cudaSuccess) return fail(PG_ERR_CUDA, cudaGetErrorString(e));
    return PG_OK;
}

int pg_get_efield_cg1(pg_sim *s, double *E) {
    if (!s || !E) return fail(PG_ERR_ARG, "pg_get_efield_cg1: NULL argument");
    std::vector<double> e4(4 * (size_t)s->ndof);
    PG_CUDA(cudaStreamSynchronize(s->stream));
    PG_CUDA(cudaMemcpy(e4.data(), s->Ev, sizeof(double) * e4.size(), cudaMemcpyDeviceToHost));
    for (int64_t d = 0; d < s->ndof; ++d)
        for (int j = 0; j < 3; ++j) E[3 * d + j] = e4[4 * d + j];
    return PG_OK;
}

static int diag_scratch(pg_sim *s) {
    if (s->diag_a) return PG_OK;
    const size_t n = (size_t)std::max(s->ndof, s->nc);
    int rc;
    if ((rc = dalloc(s, &s->diag_a, n)) || (rc = dalloc(s, &s->diag_b, n)) || (rc = dalloc(s, &s->diag_acc, 8)) ||
        (rc = dalloc(s, &s->diag_cnt, 2 * (size_t)s->nc)))
        return rc;
    return PG_OK;
}

int pg_potential_energy(pg_sim *s, double *PE) {
    if (!s || !PE) return fail(PG_ERR_ARG, "pg_potential_energy: NULL argument");
    int rc = diag_scratch(s);
    if (rc) return rc;
    launch_potential_energy(s->dm, s->P[s->cur], s->n_slots, is_mixed(s), s->d_q, s->phi, s->diag_acc, s->stream);
    PG_CUDA(cudaMemcpyAsync(PE, s->diag_acc, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return PG_OK;
}

int pg_density_cg1(pg_sim *s, double weight_e, double weight_i, double *ne, double *ni) {
    if (!s || !ne || !ni) return fail(PG_ERR_ARG, "pg_density_cg1: NULL argument");
    int rc = diag_scratch(s);
    if (rc) return rc;
    launch_density_cg1(s->dm, s->P[s->cur], s->n_slots, is_mixed(s), s->d_q, weight_e, weight_i, s->diag_a,
                       s->diag_b, s->stream);
    PG_CUDA(cudaMemcpyAsync(ne, s->diag_a, sizeof(double) * s->ndof, cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaMemcpyAsync(ni, s->diag_b, sizeof(double) * s->ndof, cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return PG_OK;
}

int pg_density_dg0(pg_sim *s, double weight_e, double weight_i, double *ne, double *ni) {
    if (!s || !ne || !ni) return fail(PG_ERR_ARG, "pg_density_dg0: NULL argument");
    int rc = diag_scratch(s);
    if (rc) return rc;
    launch_density_dg0(s->dm, s->P[s->cur], s->n_slots, s->d_q, s->es_vol, weight_e, weight_i, s->diag_cnt,
                       s->diag_a, s->diag_b, s->stream);
    PG_CUDA(cudaMemcpyAsync(ne, s->diag_a, sizeof(double) * s->nc, cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaMemcpyAsync(ni, s->diag_b, sizeof(double) * s->nc, cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return PG_OK;
}

int pg_statistics(pg_sim *s, double *stats) {
    if (!s || !stats) return fail(PG_ERR_ARG, "pg_statistics: NULL argument");
    int rc = diag_scratch(s);
    if (rc) return rc;
    launch_statistics(s->P[s->cur], s->n_slots, is_mixed(s), s->d_q, s->diag_acc, s->stream);
    double acc[6];
    PG_CUDA(cudaMemcpyAsync(acc, s->diag_acc, sizeof(acc), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    // mean and sample standard deviation per sign (population.h:800-801); no
    // particle of a sign: 0, 0
    const double m = acc[0], n = acc[2];
    stats[0] = m > 0 ? acc[1] / m : 0.0;
    stats[1] = m > 0 ? std::sqrt(acc[4] / (m - 1)) : 0.0;
    stats[2] = n > 0 ? acc[3] / n : 0.0;
    stats[3] = n > 0 ? std::sqrt(acc[5] / (n - 1)) : 0.0;
    return PG_OK;
}

// The mixed form's step forms the DG0 field inside the particle pass, from
// the potential at each particle's cell; the FP64 field (and the FP32 array
// of pg_efield_dg0) are formed from phi and these E0 when asked for.
static void pass_field(pg_sim *s, MixedParams &xp, const double E0[3]) {
    xp.phi = s->phi;
    for (int j = 0; j < 3; ++j) xp.E0[j] = (float)E0[j];
    s->E64_stale = true;
    for (int j = 0; j < 3; ++j) s->E0_last[j] = E0[j];
}

// The FP64 form's step field: the field kernel (the FP64 pass is bound by
// FP64 issue, so forming the field per particle in the pass costs as much as
// this per-cell kernel).
static void step_field_f64(pg_sim *s, const double E0[3]) {
    launch_efield(s->dm, s->phi, E0, s->stream);
    s->E64_stale = false;
}

int pg_efield_dg0(pg_sim *s, const double *phi) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    if (phi) {
        PG_CUDA(cudaMemcpyAsync(s->phi, phi, sizeof(double) * s->ndof, cudaMemcpyHostToDevice, s->stream));
        s->phi_valid = true;
    }
    const double E0[3] = {0, 0, 0};
    launch_efield(s->dm, s->phi, E0, s->stream);
    s->E64_stale = false;
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return PG_OK;
}

int pg_set_efield(pg_sim *s, const double *E) {
    if (!s || !E) return fail(PG_ERR_ARG, "pg_set_efield: NULL argument");
    std::vector<double> e4(4 * (size_t)s->nc, 0.0);
    for (int64_t c = 0; c < s->nc; ++c)
        for (int j = 0; j < 3; ++j) e4[4 * c + j] = E[3 * c + j];
    PG_CUDA(cudaMemcpy(s->dm.E, e4.data(), sizeof(double) * e4.size(), cudaMemcpyHostToDevice));
    return PG_OK;
}

int pg_get_efield(pg_sim *s, double *E) {
    if (!s || !E) return fail(PG_ERR_ARG, "pg_get_efield: NULL argument");
    std::vector<double> e4(4 * (size_t)s->nc);
    if (s->E64_stale) {
        launch_efield(s->dm, s->phi, s->E0_last, s->stream);
        s->E64_stale = false;
    }
    PG_CUDA(cudaStreamSynchronize(s->stream));
    PG_CUDA(cudaMemcpy(e4.data(), s->dm.E, sizeof(double) * e4.size(), cudaMemcpyDeviceToHost));
    for (int64_t c = 0; c < s->nc; ++c)
        for (int j = 0; j < 3; ++j) E[3 * c + j] = e4[4 * c + j];
    return PG_OK;
}

static int push_common(pg_sim *s, const double *B, double dt, bool accel, double *KE, bool cg1 = false) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    PushParams pp;
    fill_push(s, pp, dt, B, accel);
    pp.cg1 = cg1 ? 1 : 0;
    if (s->n_slots > 0) {
        if (is_mixed(s)) {
            MixedParams mp;
            fill_mixed(s, mp, dt, B, accel, 0.0, false, nullptr);
            mp.cg1 = cg1 ? 1 : 0;
            launch_mixed_pass(s->dm, s->P[s->cur], s->n_slots, mp, true, false, false, false, s->cfg.max_walk_steps,
                              s->rho_fixed, s->state, s->partials, s->n_part, s->ke_dev, s->stream);
        } else {
            launch_push(s->dm, s->P[s->cur], s->n_slots, pp, s->partials, s->n_part, s->ke_dev, s->stream);
        }
        double ke = 0;
        PG_CUDA(cudaMemcpyAsync(&ke, s->ke_dev, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        PG_CUDA(cudaStreamSynchronize(s->stream));
        if (KE) *KE = ke;
    } else if (KE) {
        *KE = 0.0;
    }
    return PG_OK;
}

int pg_accel(pg_sim *s, double dt, double *KE) { return push_common(s, nullptr, dt, true, KE); }
int pg_boris(pg_sim *s, const double B[3], double dt, double *KE) { return push_common(s, B, dt, false, KE); }
int pg_accel_cg1(pg_sim *s, double dt, double *KE) { return push_common(s, nullptr, dt, true, KE, true); }
int pg_boris_cg1(pg_sim *s, const double B[3], double dt, double *KE) { return push_common(s, B, dt, false, KE, true); }

static void move_mixed(pg_sim *s, double dt, bool periodic, const double *Ld) {
    MixedParams mp;
    fill_mixed(s, mp, 0.0, nullptr, false, dt, periodic, Ld);
    launch_mixed_pass(s->dm, s->P[s->cur], s->n_slots, mp, false, true, false, false, s->cfg.max_walk_steps,
                      s->rho_fixed, s->state, s->partials, s->n_part, s->ke_dev, s->stream);
}

int pg_move(pg_sim *s, double dt) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    MoveParams mp{};
    mp.dt = dt;
    if (s->n_slots > 0 && is_mixed(s)) move_mixed(s, dt, false, nullptr);
    else if (s->n_slots > 0) launch_move(s->P[s->cur], s->n_slots, mp, s->stream);
    PG_CUDA(cudaStreamSynchronize(s->stream));
    s->rho_valid = false;
    return PG_OK;
}

int pg_move_periodic(pg_sim *s, double dt, const double Ld[3]) {
    if (!s || !Ld) return fail(PG_ERR_ARG, "pg_move_periodic: NULL argument");
    MoveParams mp{};
    mp.dt = dt;
    mp.periodic = 1;
    for (int j = 0; j < 3; ++j) mp.Ld[j] = Ld[j];
    if (s->n_slots > 0 && is_mixed(s)) move_mixed(s, dt, true, Ld);
    else if (s->n_slots > 0) launch_move(s->P[s->cur], s->n_slots, mp, s->stream);
    PG_CUDA(cudaStreamSynchronize(s->stream));
    s->rho_valid = false;
    return PG_OK;
}

int pg_update(pg_sim *s, pg_object *objects, int32_t n_objects, double dt) {
    if (!s || (n_objects > 0 && !objects)) return fail(PG_ERR_ARG, "pg_update: bad arguments");
    PG_CUDA(cudaMemsetAsync(s->state->absorbed, 0, sizeof(s->state->absorbed), s->stream));
    if (s->n_slots > 0 && is_mixed(s)) {
        MixedParams mp;
        fill_mixed(s, mp, 0.0, nullptr, false, 0.0, false, nullptr);
        launch_mixed_pass(s->dm, s->P[s->cur], s->n_slots, mp, false, false, true, false, s->cfg.max_walk_steps,
                          s->rho_fixed, s->state, s->partials, s->n_part, s->ke_dev, s->stream);
    } else if (s->n_slots > 0) {
        launch_update(s->dm, s->P[s->cur], s->n_slots, s->cfg.max_walk_steps, s->state, s->stream);
    }
    int rc = check_state(s);
    s->rho_valid = false;
    if (rc) return rc;
    absorbed_to_objects(s, objects, n_objects, dt, nullptr);
    return PG_OK;
}

int pg_absorbed_counts(pg_sim *s, int64_t *counts, int32_t n_tags, int32_t n_species, double *q, double *m,
                       int32_t *n_species_out) {
    if (!s || n_tags < 0 || n_tags > kMaxTags || n_species < 0)
        return fail(PG_ERR_ARG, "pg_absorbed_counts: bad arguments");
    if (n_species_out) *n_species_out = s->n_species;
    if (counts && n_tags > 0 && n_species > 0) {
        int64_t tally[kMaxTags][kMaxSpecies];
        PG_CUDA(cudaStreamSynchronize(s->stream));
        PG_CUDA(cudaMemcpy(tally, s->state->absorbed, sizeof(tally), cudaMemcpyDeviceToHost));
        for (int t = 0; t < n_tags; ++t)
            for (int k = 0; k < n_species; ++k) counts[(size_t)t * n_species + k] = k < kMaxSpecies ? tally[t][k] : 0;
    }
    for (int k = 0; k < n_species; ++k) {
        if (q) q[k] = k < s->n_species ? s->q[k] : 0.0;
        if (m) m[k] = k < s->n_species ? s->m[k] : 0.0;
    }
    return PG_OK;
}

int pg_kinetic_energy(pg_sim *s, double *KE) {
    if (!s || !KE) return fail(PG_ERR_ARG, "pg_kinetic_energy: NULL argument");
    double hm[kMaxSpecies] = {0};
    for (int k = 0; k < s->n_species; ++k) hm[k] = 0.5 * s->m[k];
    *KE = 0.0;
    if (s->n_slots == 0) return PG_OK;
    if (is_mixed(s)) {
        MixedParams mp;
        fill_mixed(s, mp, 0.0, nullptr, false, 0.0, false, nullptr);
        launch_kinetic_mixed(s->P[s->cur], s->n_slots, mp, s->partials, s->n_part, s->ke_dev, s->stream);
    } else {
        launch_kinetic(s->P[s->cur], s->n_slots, hm, s->partials, s->n_part, s->ke_dev, s->stream);
    }
    PG_CUDA(cudaMemcpyAsync(KE, s->ke_dev, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return PG_OK;
}

int pg_distribute_cg1(pg_sim *s, double *rho) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    int rc = deposit_all(s);
    if (rc) return rc;
    if (rho) PG_CUDA(cudaMemcpyAsync(rho, s->rho, sizeof(double) * s->ndof, cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return PG_OK;
}

int pg_set_rho(pg_sim *s, const double *rho) {
    if (!s || !rho) return fail(PG_ERR_ARG, "pg_set_rho: NULL argument");
    PG_CUDA(cudaMemcpy(s->rho, rho, sizeof(double) * s->ndof, cudaMemcpyHostToDevice));
    s->rho_valid = false;
    return PG_OK;
}

int pg_get_rho(pg_sim *s, double *rho) {
    if (!s || !rho) return fail(PG_ERR_ARG, "pg_get_rho: NULL argument");
    PG_CUDA(cudaStreamSynchronize(s->stream));
    PG_CUDA(cudaMemcpy(rho, s->rho, sizeof(double) * s->ndof, cudaMemcpyDeviceToHost));
    return PG_OK;
}

int pg_get_phi(pg_sim *s, double *phi) {
    if (!s || !phi) return fail(PG_ERR_ARG, "pg_get_phi: NULL argument");
    PG_CUDA(cudaStreamSynchronize(s->stream));
    PG_CUDA(cudaMemcpy(phi, s->phi, sizeof(double) * s->ndof, cudaMemcpyDeviceToHost));
    return PG_OK;
}

// The potential as it stands after the work queued so far: copied to a
// device snapshot on the engine stream, then read back to phi on a copy
// stream, so the next steps run while the copy is in flight.  The snapshot is
// written again only after the previous read-back has finished.
int pg_get_phi_async(pg_sim *s, double *phi) {
    if (!s || !phi) return fail(PG_ERR_ARG, "pg_get_phi_async: NULL argument");
    if (!s->phi_snap) {
        const int rc = dalloc(s, &s->phi_snap, s->ndof);
        if (rc) return rc;
    }
    if (!s->copy_stream) PG_CUDA(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
    if (!s->phi_ready) PG_CUDA(cudaEventCreateWithFlags(&s->phi_ready, cudaEventDisableTiming));
    if (!s->phi_copied) PG_CUDA(cudaEventCreateWithFlags(&s->phi_copied, cudaEventDisableTiming));
    if (s->phi_copy_pending) PG_CUDA(cudaStreamWaitEvent(s->stream, s->phi_copied, 0));
    PG_CUDA(cudaMemcpyAsync(s->phi_snap, s->phi, sizeof(double) * s->ndof, cudaMemcpyDeviceToDevice, s->stream));
    PG_CUDA(cudaEventRecord(s->phi_ready, s->stream));
    PG_CUDA(cudaStreamWaitEvent(s->copy_stream, s->phi_ready, 0));
    PG_CUDA(cudaMemcpyAsync(phi, s->phi_snap, sizeof(double) * s->ndof, cudaMemcpyDeviceToHost, s->copy_stream));
    PG_CUDA(cudaEventRecord(s->phi_copied, s->copy_stream));
    s->phi_copy_pending = true;
    return PG_OK;
}

int pg_poisson_solve(pg_sim *s, const pg_object *objects, int32_t n_objects, double *phi, pg_solve_info *info) {
    if (!s || (n_objects > 0 && !objects)) return fail(PG_ERR_ARG, "pg_poisson_solve: bad arguments");
    std::vector<double> pot(std::max(1, s->n_obj), 0.0);
    for (int k = 0; k < n_objects; ++k) {
        const int i = object_index(s, objects[k].bnd_id);
        if (i < 0) return fail(PG_ERR_ARG, "object bnd_id is not an object tag");
        pot[i] = objects[k].potential;
    }
    pg_solve_info acc{};
    int rc = poisson_solve_internal(s, pot.data(), false, true, s->cfg.pcg_rtol, s->cfg.pcg_atol, &acc);
    if (info) *info = acc;
    if (rc) return rc;
    if (phi) return pg_get_phi(s, phi);
    return PG_OK;
}

int pg_circuit_cm_setup(pg_sim *s, const pg_source *vs, int32_t nvs, const pg_source *is, int32_t nis, double dt) {
    if (!s || (nvs > 0 && !vs) || (nis > 0 && !is)) return fail(PG_ERR_ARG, "pg_circuit_cm_setup: bad arguments");
    const int n = s->n_obj;
    if (n == 0) return fail(PG_ERR_STATE, "pg_circuit_cm_setup: the mesh has no objects");
    for (int k = 0; k < nvs; ++k)
        if (vs[k].node_b < 0 || vs[k].node_b >= n || vs[k].node_a < -1 || vs[k].node_a >= n)
            return fail(PG_ERR_ARG, "voltage source node out of range");
    for (int k = 0; k < nis; ++k)
        if (is[k].node_b < -1 || is[k].node_b >= n || is[k].node_a < -1 || is[k].node_a >= n)
            return fail(PG_ERR_ARG, "current source node out of range");
    s->vsrc.assign(vs, vs + nvs);
    s->isrc.assign(is, is + nis);
    s->circ_dt = dt;
    // capacitance matrix: one Laplace solve per object (inv_capacitance,
    // punc/src/object_CM.cpp:62-106 and laplace_solver 401-437).
    std::vector<double> cap(n * n, 0.0);
    std::vector<int32_t> rng(2 * (size_t)n, 0);
    if (!s->lap) {
        int rc = dalloc(s, &s->lap, (size_t)n * s->ndof);
        if (rc) return rc;
    }
    for (int j = 0; j < n; ++j) {
        std::vector<double> pot(n, 0.0);
        pot[j] = 1.0;
        // the reference's laplace_solver uses the PoissonSolver defaults (rel 1e-12, abs 1e-14)
        int rc = poisson_solve_internal(s, pot.data(), true, false, std::min(1e-12, s->cfg.pcg_rtol),
                                        std::min(1e-14, s->cfg.pcg_atol), nullptr);
        if (rc) return rc;
        std::vector<double> img;
        rc = image_charges(s, img);
        if (rc) return rc;
        for (int i = 0; i < n; ++i) cap[i * n + j] = img[i];
        PG_CUDA(cudaMemcpyAsync(s->lap + (size_t)j * s->ndof, s->phi, sizeof(double) * s->ndof,
                                cudaMemcpyDeviceToDevice, s->stream));
        // the dof range of L_j's entries above 1e-12 of its largest: the
        // superposition skips the rest (in batched runs L_j lives in its run)
        std::vector<double> h((size_t)s->ndof);
        PG_CUDA(cudaMemcpyAsync(h.data(), s->phi, sizeof(double) * s->ndof, cudaMemcpyDeviceToHost, s->stream));
        PG_CUDA(cudaStreamSynchronize(s->stream));
        double vmax = 0.0;
        for (double v : h) vmax = std::max(vmax, std::fabs(v));
        int32_t lo = s->ndof, hi = 0;
        for (int32_t i = 0; i < s->ndof; ++i)
            if (std::fabs(h[i]) > 1e-12 * vmax) { lo = std::min(lo, i); hi = i + 1; }
        rng[2 * j] = lo < hi ? lo : 0;
        rng[2 * j + 1] = hi;
    }
    if (!s->lap_rng) {
        int rc = dalloc(s, &s->lap_rng, 2 * (size_t)n);
        if (rc) return rc;
    }
    PG_CUDA(cudaMemcpyAsync(s->lap_rng, rng.data(), sizeof(int32_t) * 2 * n, cudaMemcpyHostToDevice, s->stream));
    s->phi0_valid = false;
    s->phi_valid = false;
    s->inv_cap = cap;
    if (!invert(s->inv_cap, n)) return fail(PG_ERR_SINGULAR, "capacitance matrix is singular");
    // circuit matrix (CircuitCM::CircuitCM and assemble_matrix, object_CM.cpp:135-273)
    s->groups = charge_sharing_sets(s->vsrc, n);
    s->fixed_voltage.clear();
    for (size_t i = 0; i < s->vsrc.size(); ++i) {
        if (s->vsrc[i].node_a == -1) {
            std::vector<int> tmp{s->vsrc[i].node_b};
            int node = s->vsrc[i].node_b;
            for (size_t j = 0; j < s->vsrc.size(); ++j)
                if (s->vsrc[j].node_a == node) { tmp.push_back(s->vsrc[j].node_b); node = s->vsrc[j].node_b; }
            s->fixed_voltage.push_back(tmp);
        }
    }
    s->circ_vec.assign(2 * n, 0.0);
    for (auto &v : s->vsrc) s->circ_vec[v.node_b] = v.value;
    std::vector<double> cm(4 * n * n, 0.0);
    auto C = [&](int r, int c) -> double & { return cm[r * 2 * n + c]; };
    auto IC = [&](int r, int c) { return s->inv_cap[r * n + c]; };
    for (auto &v : s->vsrc) {
        C(v.node_b, v.node_b) = 1.0;
        if (v.node_a != -1) C(v.node_b, v.node_a) = -1.0;
    }
    for (auto &g : s->groups) {
        for (int v : g) C(n + g[0], n + v) = 1.0;
        C(g[0], g[0]) = 1.0;
        for (int v : g) C(g[0], n + v) = -1.0 * IC(g[0], v);
        for (size_t j = 1; j < g.size(); ++j) {
            C(n + g[j], g[j]) = 1.0;
            for (int v : g) C(n + g[j], n + v) = -1.0 * IC(g[j], v);
        }
    }
    for (auto &fv : s->fixed_voltage)
        for (int a : fv) {
            C(n + a, a) = 1.0;
            for (int b : fv) C(n + a, n + b) = -1.0 * IC(a, b);
        }
    s->inv_circ = cm;
    if (!invert(s->inv_circ, 2 * n)) return fail(PG_ERR_SINGULAR, "circuit matrix is singular");
    s->circuit_ready = true;
    return PG_OK;
}

int pg_get_capacitance(pg_sim *s, double *inv_cap) {
    if (!s || !inv_cap) return fail(PG_ERR_ARG, "pg_get_capacitance: NULL argument");
    if (!s->circuit_ready) return fail(PG_ERR_STATE, "circuit not set up");
    std::copy(s->inv_cap.begin(), s->inv_cap.end(), inv_cap);
    return PG_OK;
}

int pg_solve_circuit(pg_sim *s, pg_object *objects, int32_t n_objects, double *phi, pg_solve_info *info) {
    if (!s || (n_objects > 0 && !objects)) return fail(PG_ERR_ARG, "pg_solve_circuit: bad arguments");
    if (!s->circuit_ready) return fail(PG_ERR_STATE, "pg_solve_circuit: call pg_circuit_cm_setup first");
    pg_solve_info acc{};
    int rc = solve_circuit_internal(s, objects, n_objects, &acc);
    if (info) *info = acc;
    if (rc) return rc;
    if (phi) return pg_get_phi(s, phi);
    return PG_OK;
}

int pg_create_flux(pg_sim *s, const pg_species *sp, int32_t n) {
    if (!s || (n > 0 && !sp) || n < 0 || n > kMaxSpecies) return fail(PG_ERR_ARG, "pg_create_flux: bad arguments");
    // Species slots follow the engine's species ids; injection table rows are
    // indexed by engine species id so particles carry consistent ids.
    pg_species tab[kMaxSpecies]{};
    int nmax = 0;
    for (int k = 0; k < n; ++k) {
        const int id = species_id(s, sp[k].q, sp[k].m);
        if (id < 0) return fail(PG_ERR_ARG, "pg_create_flux: more than 8 species");
        tab[id] = sp[k];
        nmax = std::max(nmax, id + 1);
    }
    const int nf = s->n_ext;
    std::vector<double> num((size_t)nmax * nf, 0.0), pmax((size_t)nmax * nf, 0.0);
    for (int k = 0; k < nmax; ++k) {
        const pg_species &S = tab[k];
        if (S.vth <= 0 && S.n == 0) continue;   // species without inflow
        const double vth = S.vth, vth2 = vth * vth;
        const double factor = 1.0 / std::pow(std::sqrt(2. * M_PI * vth2), 3);
        for (int j = 0; j < nf; ++j) {
            const double *F = &s->ext_facets_h[14 * (size_t)j];
            const double area = F[0];
            const double nrm[3] = {F[10], F[11], F[12]};
            // Maxwellian::flux_num_particles (punc/src/distributions.cpp:52-60)
            double vdn = 0.0;
            for (int c = 0; c < 3; ++c) vdn += nrm[c] * S.vd[c];
            num[(size_t)k * nf + j] = area * (vth / (std::sqrt(2 * M_PI)) * std::exp(-0.5 * (vdn / vth) * (vdn / vth)) +
                                             0.5 * vdn * (1. + std::erf(vdn / (std::sqrt(2) * vth))));
            // Maxwellian::flux_max (punc/src/distributions.cpp:62-72)
            double tmp[3];
            for (int c = 0; c < 3; ++c) tmp[c] = S.vd[c] - 0.5 * nrm[c] * vdn + 0.5 * nrm[c] * std::sqrt(4 * vth2 + vdn * vdn);
            double vn = 0.0;
            for (int c = 0; c < 3; ++c) vn += tmp[c] * nrm[c];
            double vsq = 0.0;
            for (int c = 0; c < 3; ++c) vsq += (tmp[c] - S.vd[c]) * (tmp[c] - S.vd[c]);
            pmax[(size_t)k * nf + j] = (vn > 0.0) * vn * (factor * std::exp(-0.5 * vsq / vth2));
        }
    }
    if (s->flux_num) cudaFree(s->flux_num);
    if (s->pdf_max) cudaFree(s->pdf_max);
    if (s->inj_counts) cudaFree(s->inj_counts);
    if (s->inj_offsets) cudaFree(s->inj_offsets);
    s->flux_num = s->pdf_max = nullptr;
    s->inj_counts = s->inj_offsets = nullptr;
    const size_t tot = std::max<size_t>(1, (size_t)nmax * nf);
    PG_CUDA(cudaMalloc(&s->flux_num, sizeof(double) * tot));
    PG_CUDA(cudaMalloc(&s->pdf_max, sizeof(double) * tot));
    PG_CUDA(cudaMalloc(&s->inj_counts, sizeof(int64_t) * (tot + 1)));
    PG_CUDA(cudaMalloc(&s->inj_offsets, sizeof(int64_t) * (tot + 1)));
    if (!num.empty()) {
        PG_CUDA(cudaMemcpy(s->flux_num, num.data(), sizeof(double) * num.size(), cudaMemcpyHostToDevice));
        PG_CUDA(cudaMemcpy(s->pdf_max, pmax.data(), sizeof(double) * pmax.size(), cudaMemcpyHostToDevice));
    }
    s->flux_num_h = num;
    s->flux_sum_h.assign(nmax, 0.0);
    for (int k = 0; k < nmax; ++k)
        for (int64_t j = 0; j < nf; ++j) s->flux_sum_h[k] += num[(size_t)k * nf + j];
    s->n_inj_species = nmax;
    for (int k = 0; k < nmax; ++k) s->inj[k] = tab[k];
    s->flux_ready = true;
    return PG_OK;
}

int pg_inject(pg_sim *s, double dt, uint64_t seed, uint64_t step, int64_t *n_injected) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    int rc = inject_internal(s, dt, seed, step, false, n_injected);
    s->rho_valid = false;
    return rc;
}

int pg_sort(pg_sim *s) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    return do_sort(s);
}

// ---- multi-step runs: the step on the device only ------------------------

// rhs, boundary values and one PCG launch into x; object potentials are read
// from s->obj_pot on the device; no status read-back.
static int pcg_enqueue(pg_sim *s, double *x) {
    launch_rhs(s->dm, s->Ms_ptr, s->Ms_width, s->Ms_col, s->Ms_val, s->rho, s->bc_kind, s->bc_value, s->w_ext, s->w_obj, s->obj_pot,
               s->n_obj, 1, s->b, s->stream);
    launch_set_bc(s->bc_kind, s->bc_value, s->obj_pot, s->ndof, x, s->stream);
    PcgArgs a{};
    a.n = s->ndof;
    a.slice_ptr = s->A_sptr; a.slice_width = s->A_swidth; a.col = s->A_col; a.val = s->A_val; a.dinv = s->A_dinv;
    a.b = s->b; a.x = x; a.r = s->r; a.z = s->z; a.p0 = s->p0; a.p1 = s->p1; a.Ap = s->Ap;
    a.partials = s->pcg_part;
    a.rtol = s->cfg.pcg_rtol; a.atol = s->cfg.pcg_atol;
    a.max_iter = s->cfg.pcg_max_iter;
    a.remove_mean = s->cfg.periodic ? 1 : 0;
    a.out_iter = s->pcg_out_i; a.out_status = s->pcg_out_i + 1;
    a.out_rr = s->pcg_out_d; a.out_bb = s->pcg_out_d + 1;
    a.val32 = s->A_val32; a.dinv32 = s->A_dinv32;
    a.r32 = s->r32; a.z32 = s->z32; a.p32 = s->p32; a.Ap32 = s->Ap32;
    a.out_updates = nullptr;
    const int e = s->use_amg ? launch_pcg_amg(a, s->amg, s->stream) : launch_pcg(a, s->stream);
    if (e) return fail(PG_ERR_CUDA, std::string("cooperative PCG launch: ") + cudaGetErrorString((cudaError_t)e));
    return PG_OK;
}

// Per-step injection bound: sum over species of ceil(n dt sum_j flux_j) + facets.
static int64_t inject_bound(const pg_sim *s, double dt) {
    int64_t bound = 0;
    for (int k = 0; k < s->n_inj_species; ++k)
        bound += (int64_t)std::ceil(s->flux_sum_h[k] * s->inj[k].n * dt) + s->n_ext;
    return bound;
}

// Injection with the slot base, id base and RNG step read from run_counts,
// depositing into this step's accumulator; counters advanced on the device.
static void inject_enqueue(pg_sim *s, const DevParticles &Pd, double dt, uint64_t seed) {
    const int total = s->n_inj_species * s->n_ext;
    if (total == 0) return;
    InjectParams ip{};
    ip.n_species = s->n_inj_species;
    ip.n_facets = s->n_ext;
    ip.seed = seed;
    ip.dt = dt;
    for (int k = 0; k < s->n_inj_species; ++k) {
        const pg_species &S = s->inj[k];
        InjectSpecies &I = ip.sp[k];
        I.ndt = S.n * dt;
        const double range = S.vdf_range > 0 ? S.vdf_range : 5.0;
        for (int c = 0; c < 3; ++c) {
            const double lo = S.vd[c] - range * S.vth, hi = S.vd[c] + range * S.vth;
            I.domain_lo[c] = lo;
            I.domain_w[c] = hi - lo;
            I.vd[c] = S.vd[c];
        }
        I.vth2 = S.vth * S.vth;
        I.factor = 1.0 / std::pow(std::sqrt(2. * M_PI * I.vth2), 3);
        I.q = S.q;
    }
    fill_flux32(ip);
    ip.facets_f = s->d_ext_facets_f;
    ip.counts_dev = s->run_counts;
    ip.facet_c1 = s->d_inj_c1;
    ip.facet_seed = s->d_inj_seed;
    ip.rho_fixed = s->rho_fixed;
    const double unit = fixed_unit(s);
    for (int k = 0; k < s->n_species; ++k) ip.q_scaled[k] = (float)(s->q[k] / unit);
    cudaMemsetAsync(s->inj_counts, 0, sizeof(int64_t) * (total + 1), s->stream);
    cudaMemsetAsync(s->state->injected, 0, sizeof(s->state->injected), s->stream);
    launch_inject_count(s->dm, ip, s->flux_num, s->inj_counts, s->stream);
    launch_scan_i64(s->inj_counts, s->inj_offsets, total + 1, s->scan_tmp, s->stream);
    launch_inject_generate(s->dm, Pd, ip, s->flux_num, s->pdf_max, s->d_ext_facets, s->inj_offsets,
                           s->cfg.max_walk_steps, 1, s->d_q, s->rho_acc, s->state, inject_bound(s, dt), s->stream);
    launch_inject_commit(s->run_counts, s->state, s->stream);
}

// One whole step on the stream, no host synchronisation: the same operations
// and arithmetic as pg_step, with counts, objects and the circuit on the device.
static int enqueue_step(pg_sim *s, const pg_step_args *a, bool first) {
    DevParticles Pd = s->P[s->cur];
    Pd.n_dev = s->run_counts;
    const int64_t cap = Pd.capacity;
    rho_from_acc(s);
    int rc;
    if (s->circuit_ready) {
        launch_circuit_pre(s->run_isrc, (int)s->isrc.size(), s->circ_dt, s->n_obj, s->run_obj, s->obj_pot, s->stream);
        const bool superpose = !s->cfg.circuit_resolve && s->lap;
        if ((rc = pcg_enqueue(s, superpose ? s->phi0 : s->phi))) return rc;
        launch_image_charge(s->dm, superpose ? s->phi0 : s->phi, s->d_ofacets, s->n_ofac, s->n_obj, s->cfg.eps0,
                            s->image, s->stream);
        launch_circuit_post(s->circ_dev, s->image, s->run_obj, s->obj_pot, s->stream);
        if (superpose) launch_superpose_dev(s->phi0, s->lap, s->obj_pot, s->lap_rng, s->n_obj, s->ndof, s->phi, s->stream);
        else if ((rc = pcg_enqueue(s, s->phi))) return rc;
    } else {
        if ((rc = pcg_enqueue(s, s->phi))) return rc;
    }
    if (a->efield_cg1) {
        EsolveArgs e{};
        const double zero[3] = {0, 0, 0};
        launch_efield(s->dm, s->phi, zero, s->stream);
        e.n = s->ndof;
        e.fp32 = is_mixed(s) ? 1 : 0;
        e.adj_ptr = s->es_adj_ptr; e.adj_cell = s->es_adj_cell; e.vol = s->es_vol; e.E_cell = s->dm.E;
        e.row = s->M_row; e.col = s->M_col; e.val = s->M_val; e.dinv = s->M_dinv;
        e.val32 = s->M_val32; e.dinv32 = s->M_dinv32;
        const size_t n3 = 3 * (size_t)s->ndof;
        if (e.fp32) {
            float *b = s->es_buf32;
            e.b32 = b; e.x32 = b + n3; e.r32 = b + 2 * n3; e.z32 = b + 3 * n3; e.p32 = b + 4 * n3; e.Ap32 = b + 5 * n3;
            e.rtol = 1e-6;
        } else {
            double *b = s->es_buf;
            e.b = b; e.x = b + n3; e.r = b + 2 * n3; e.z = b + 3 * n3; e.p = b + 4 * n3; e.Ap = b + 5 * n3;
            e.rtol = 1e-12;
        }
        e.atol = 1e-14;
        e.max_iter = 1000;
        e.partials = s->es_part;
        e.out_iter = s->es_out_i; e.out_status = s->es_out_i + 1;
        e.out_rr = s->es_out_d; e.out_bb = s->es_out_d + 3;
        for (int j = 0; j < 3; ++j) e.E0[j] = a->E0[j];
        e.ev = s->Ev;
        e.evf = s->Evf;
        const int err = launch_esolve(e, s->stream);
        if (err) return fail(PG_ERR_CUDA, std::string("ESolver launch: ") + cudaGetErrorString((cudaError_t)err));
    } else if (!is_mixed(s)) {
        step_field_f64(s, a->E0);
    }
    const double dt_push = first ? 0.5 * a->dt : a->dt;
    cudaMemsetAsync(s->state->absorbed, 0, sizeof(s->state->absorbed), s->stream);
    if (is_mixed(s)) {
        cudaMemsetAsync(s->rho_fixed, 0, sizeof(unsigned long long) * s->ndof, s->stream);
        MixedParams xp;
        fill_mixed(s, xp, dt_push, a->B, a->use_accel != 0, a->dt, a->periodic_move != 0, a->Ld);
        xp.cg1 = a->efield_cg1 ? 1 : 0;
        if (!a->efield_cg1) pass_field(s, xp, a->E0);
        launch_mixed_pass(s->dm, Pd, cap, xp, true, true, true, true, s->cfg.max_walk_steps, s->rho_fixed, s->state,
                          s->partials, s->n_part, s->ke_dev, s->stream);
    } else {
        cudaMemsetAsync(s->rho_acc, 0, sizeof(double) * s->ndof, s->stream);
        PushParams pp;
        fill_push(s, pp, dt_push, a->B, a->use_accel != 0);
        pp.cg1 = a->efield_cg1 ? 1 : 0;
        MoveParams mp{};
        mp.dt = a->dt;
        mp.periodic = a->periodic_move;
        for (int j = 0; j < 3; ++j) mp.Ld[j] = a->Ld[j];
        launch_fused_step(s->dm, Pd, cap, pp, mp, s->cfg.max_walk_steps, s->d_q, s->rho_acc, s->state, s->partials,
                          s->n_part, s->ke_dev, s->stream);
    }
    launch_objects_update(s->state, s->d_q, s->n_species, s->run_tags, s->n_obj, s->run_obj, a->dt, s->stream);
    if (a->inject) inject_enqueue(s, Pd, a->dt, a->seed);
    else cudaMemsetAsync(s->state->injected, 0, sizeof(s->state->injected), s->stream);
    launch_step_record(s->run_rows, 6 + 3 * s->n_obj, s->run_counts, s->ke_dev, s->state, s->n_species, s->pcg_out_i,
                       s->pcg_out_d, s->run_obj, s->n_obj, s->stream);
    return PG_OK;
}

// Cell sort on the device with the counts of a run (no read-back).
static void sort_enqueue(pg_sim *s) {
    const int other = 1 - s->cur;
    DevParticles Pd = s->P[s->cur];
    Pd.n_dev = s->run_counts;
    cudaMemsetAsync(s->sort_hist, 0, sizeof(int64_t) * (s->nc + 1), s->stream);
    launch_sort_hist(Pd, Pd.capacity, s->sort_hist, s->stream);
    launch_scan_i64(s->sort_hist, s->sort_cursor, s->nc + 1, s->scan_tmp, s->stream);
    launch_sort_scatter(Pd, s->P[other], Pd.capacity, s->sort_cursor, s->stream);
    launch_set_count(s->run_counts, s->sort_cursor, s->nc, s->stream);
    s->cur = other;
}

static void drop_graphs(pg_sim *s) {
    for (int k = 0; k < 2; ++k) {
        if (s->graph_exec[k]) cudaGraphExecDestroy(s->graph_exec[k]);
        s->graph_exec[k] = nullptr;
        s->graph_key[k].clear();
    }
}

// Device copies of the circuit matrices and groups (once per circuit set-up).
static int upload_circuit(pg_sim *s) {
    if (s->circ_dev_ready || !s->circuit_ready) return PG_OK;
    const int n = s->n_obj;
    std::vector<int32_t> gp{0}, gm, fp{0}, fm;
    for (auto &g : s->groups) { for (int v : g) gm.push_back(v); gp.push_back((int32_t)gm.size()); }
    for (auto &f : s->fixed_voltage) { for (int v : f) fm.push_back(v); fp.push_back((int32_t)fm.size()); }
    int32_t *d_gp, *d_gm, *d_fp, *d_fm;
    double *d_ic, *d_icc, *d_cv;
    int rc;
    if ((rc = upload(s, &d_gp, gp)) || (rc = upload(s, &d_gm, gm)) || (rc = upload(s, &d_fp, fp)) ||
        (rc = upload(s, &d_fm, fm)) || (rc = upload(s, &d_ic, s->inv_cap)) || (rc = upload(s, &d_icc, s->inv_circ)) ||
        (rc = upload(s, &d_cv, s->circ_vec)))
        return rc;
    CircuitDev &c = s->circ_dev;
    c.n = n;
    c.n_groups = (int32_t)s->groups.size();
    c.n_fv = (int32_t)s->fixed_voltage.size();
    c.g_ptr = d_gp; c.g_mem = d_gm; c.f_ptr = d_fp; c.f_mem = d_fm;
    c.inv_cap = d_ic; c.inv_circ = d_icc; c.cv = d_cv;
    std::vector<double> isrc;
    for (auto &x : s->isrc) { isrc.push_back(x.node_a); isrc.push_back(x.node_b); isrc.push_back(x.value); }
    if ((rc = upload(s, &s->run_isrc, isrc))) return rc;
    s->circ_dev_ready = true;
    return PG_OK;
}

int pg_run_steps(pg_sim *s, const pg_step_args *a, pg_object *objects, int32_t n_objects, int32_t n_steps,
                 int32_t use_graph, pg_step_result *results) {
    if (!s || !a || n_steps < 0 || (n_objects > 0 && !objects)) return fail(PG_ERR_ARG, "pg_run_steps: bad arguments");
    if (a->potential_energy)
        return fail(PG_ERR_ARG, "pg_run_steps: the potential energy is computed per step by pg_step only");
    if (n_steps == 0) return PG_OK;
    const int n = s->n_obj;
    std::vector<int> map(n, -1);
    for (int k = 0; k < n_objects; ++k) {
        const int i = object_index(s, objects[k].bnd_id);
        if (i >= 0) map[i] = k;
    }
    if (s->circuit_ready)
        for (int i = 0; i < n; ++i)
            if (map[i] < 0) return fail(PG_ERR_ARG, "pg_run_steps: the circuit needs every object of the mesh");
    if (a->inject && !s->flux_ready) return fail(PG_ERR_STATE, "pg_run_steps: call pg_create_flux first");
    int rc;
    if (!s->run_counts) {
        if ((rc = dalloc(s, &s->run_counts, 4)) || (rc = dalloc(s, &s->run_obj, 4 * (size_t)std::max(1, n))) ||
            (rc = dalloc(s, &s->run_tags, (size_t)std::max(1, n))))
            return rc;
        std::vector<int64_t> tags(std::max(1, n), 0);
        for (int i = 0; i < n; ++i) tags[i] = i + 2;
        PG_CUDA(cudaMemcpy(s->run_tags, tags.data(), sizeof(int64_t) * tags.size(), cudaMemcpyHostToDevice));
    }
    if ((rc = upload_circuit(s))) return rc;
    const int row_len = 6 + 3 * n;
    if (s->run_rows_cap < (int64_t)n_steps * row_len) {
        if ((rc = dalloc(s, &s->run_rows, (size_t)n_steps * row_len))) return rc;
        s->run_rows_cap = (int64_t)n_steps * row_len;
    }
    // capacity for the injections between two sorts, and scan scratch
    const int per_chunk = std::min(n_steps, std::max(1, s->cfg.sort_interval));
    const int64_t grow = a->inject ? inject_bound(s, a->dt) * per_chunk : 0;
    const int64_t cap_before = s->P[0].capacity;
    if ((rc = ensure_capacity(s, s->n_slots + grow))) return rc;
    if (s->P[0].capacity != cap_before) drop_graphs(s);
    if (a->inject && (rc = ensure_scan_tmp(s, s->n_inj_species * s->n_ext + 1))) return rc;
    // device state: counts, objects, potentials of fixed-potential objects
    const int64_t counts[4] = {s->n_slots, s->next_pid, (int64_t)a->step, 0};
    PG_CUDA(cudaMemcpyAsync(s->run_counts, counts, sizeof(counts), cudaMemcpyHostToDevice, s->stream));
    std::vector<double> obj(4 * (size_t)std::max(1, n), 0.0), pot(std::max(1, n), 0.0);
    for (int i = 0; i < n; ++i)
        if (map[i] >= 0) {
            obj[4 * i] = objects[map[i]].charge;
            obj[4 * i + 1] = objects[map[i]].current;
            obj[4 * i + 2] = objects[map[i]].potential;
            pot[i] = objects[map[i]].potential;
        }
    PG_CUDA(cudaMemcpyAsync(s->run_obj, obj.data(), sizeof(double) * obj.size(), cudaMemcpyHostToDevice, s->stream));
    if (n > 0) PG_CUDA(cudaMemcpyAsync(s->obj_pot, pot.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s->stream));
    if (!s->rho_valid && (rc = deposit_into_acc(s))) return rc;
    // the circuit solve warm-starts from phi0; the plain solve from phi
    if (!s->cfg.pcg_warm_start || !(s->circuit_ready && !s->cfg.circuit_resolve && s->lap ? s->phi0_valid : s->phi_valid))
        PG_CUDA(cudaMemsetAsync(s->circuit_ready && !s->cfg.circuit_resolve && s->lap ? s->phi0 : s->phi, 0,
                                sizeof(double) * s->ndof, s->stream));
    const bool profiling = s->profiling;
    s->profiling = false;
    const long long launches0 = launches_so_far();
    int k = 0;
    if (a->first_step) {
        if ((rc = enqueue_step(s, a, true))) { s->profiling = profiling; return rc; }
        ++k;
        ++s->step_count;
        if (s->step_count % s->cfg.sort_interval == 0) sort_enqueue(s);
    }
    // a captured step is valid for these arguments and these buffers
    pg_step_args ak = *a;
    ak.step = 0;            // read from the device counters
    ak.first_step = 0;
    std::string key(reinterpret_cast<const char *>(&ak), sizeof(pg_step_args));
    const void *bufs[] = {s->scan_tmp, s->inj_counts, s->inj_offsets, s->flux_num, s->pdf_max, s->run_rows,
                          s->d_inj_c1, s->d_inj_seed};
    key.append(reinterpret_cast<const char *>(bufs), sizeof(bufs));
    const int32_t flags[] = {s->n_inj_species, s->flux_ready ? 1 : 0, s->circuit_ready ? 1 : 0, s->n_species};
    key.append(reinterpret_cast<const char *>(flags), sizeof(flags));
    while (k < n_steps) {
        if (use_graph) {
            const int c = s->cur;
            if (!s->graph_exec[c] || s->graph_key[c] != key || s->graph_cap[c] != s->P[c].capacity) {
                if (s->graph_exec[c]) cudaGraphExecDestroy(s->graph_exec[c]);
                s->graph_exec[c] = nullptr;
                cudaGraph_t g = nullptr;
                const long long l0 = launches_so_far();
                cudaError_t e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
                if (e == cudaSuccess) {
                    rc = enqueue_step(s, a, false);
                    e = cudaStreamEndCapture(s->stream, &g);
                }
                if (e == cudaSuccess && rc == PG_OK) e = cudaGraphInstantiate(&s->graph_exec[c], g, 0);
                if (g) cudaGraphDestroy(g);
                if (e != cudaSuccess || rc != PG_OK) {
                    s->profiling = profiling;
                    s->graph_exec[c] = nullptr;
                    cudaGetLastError();
                    return rc ? rc : fail(PG_ERR_CUDA, std::string("step graph capture: ") + cudaGetErrorString(e));
                }
                s->graph_launches = launches_so_far() - l0;
                s->graph_key[c] = key;
                s->graph_cap[c] = s->P[c].capacity;
            }
            PG_CUDA(cudaGraphLaunch(s->graph_exec[c], s->stream));
            count_launches((int)s->graph_launches);
        } else if ((rc = enqueue_step(s, a, false))) {
            s->profiling = profiling;
            return rc;
        }
        ++k;
        ++s->step_count;
        if (s->step_count % s->cfg.sort_interval == 0) sort_enqueue(s);
    }
    s->profiling = profiling;
    (void)launches0;
    // read back once
    int64_t cnt[4];
    std::vector<double> rows((size_t)n_steps * row_len);
    PG_CUDA(cudaMemcpyAsync(cnt, s->run_counts, sizeof(cnt), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaMemcpyAsync(obj.data(), s->run_obj, sizeof(double) * obj.size(), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaMemcpyAsync(rows.data(), s->run_rows, sizeof(double) * rows.size(), cudaMemcpyDeviceToHost, s->stream));
    rc = check_state(s);
    s->n_slots = cnt[0];
    s->next_pid = cnt[1];
    s->rho_valid = true;
    s->phi_valid = true;
    if (s->circuit_ready && !s->cfg.circuit_resolve && s->lap) s->phi0_valid = true;
    for (int i = 0; i < n; ++i)
        if (map[i] >= 0) {
            objects[map[i]].charge = obj[4 * i];
            objects[map[i]].current = obj[4 * i + 1];
            objects[map[i]].potential = obj[4 * i + 2];
        }
    if (results)
        for (int j = 0; j < n_steps; ++j) {
            const double *r = rows.data() + (size_t)j * row_len;
            pg_step_result &o = results[j];
            o = pg_step_result{};
            o.KE = r[0];
            o.n_particles = (int64_t)r[1];
            o.n_absorbed = (int64_t)r[2];
            o.n_injected = (int64_t)r[3];
            o.pcg_iterations = (int32_t)r[4];
            o.pcg_residual = r[5];
        }
    if (rc) return rc;
    int32_t oi[2];
    PG_CUDA(cudaMemcpy(oi, s->pcg_out_i, sizeof(oi), cudaMemcpyDeviceToHost));
    if (oi[1] != 0) return fail(PG_ERR_NOT_CONVERGED, "pg_run_steps: the last PCG solve did not converge");
    return PG_OK;
}

int pg_set_tuning(pg_sim *s, const pg_tuning *t) {
    if (!s || !t) return fail(PG_ERR_ARG, "pg_set_tuning: NULL argument");
    if (t->threads != 0 && (t->threads < 32 || t->threads > 512 || (t->threads & 31)))
        return fail(PG_ERR_ARG, "pg_set_tuning: threads must be 0 or a multiple of 32 in [32, 512]");
    if (t->blocks_per_sm < 0 || sm_count() * t->blocks_per_sm > s->part_cap)
        return fail(PG_ERR_ARG, "pg_set_tuning: blocks_per_sm out of range (at most 32)");
    if (t->sort_interval < 0) return fail(PG_ERR_ARG, "pg_set_tuning: negative sort_interval");
    s->tune_threads = t->threads;
    if (t->blocks_per_sm > 0) s->n_part = sm_count() * t->blocks_per_sm;
    s->tune_dep_agg = t->dep_agg ? 1 : 0;
    if (t->sort_interval > 0) s->cfg.sort_interval = t->sort_interval;
    drop_graphs(s);
    return PG_OK;
}

int pg_get_tuning(pg_sim *s, pg_tuning *t) {
    if (!s || !t) return fail(PG_ERR_ARG, "pg_get_tuning: NULL argument");
    *t = pg_tuning{};
    t->threads = s->tune_threads ? s->tune_threads : 256;
    t->blocks_per_sm = s->n_part / sm_count();
    t->dep_agg = s->tune_dep_agg;
    t->sort_interval = s->cfg.sort_interval;
    return PG_OK;
}

// Device time of the fused particle pass of one pg_step, from the stage timer.
static double pass_ms(pg_sim *s) {
    for (size_t k = 0; k < s->stage_names.size(); ++k)
        if (s->stage_names[k] == "push_move_update_deposit") return s->stage_ms[k];
    return 0.0;
}

int pg_autotune(pg_sim *s, const pg_step_args *a, pg_object *objects, int32_t n_objects, int32_t steps_per_trial,
                pg_tuning *out) {
    if (!s || !a) return fail(PG_ERR_ARG, "pg_autotune: NULL argument");
    const int k = std::max(1, steps_per_trial);
    const bool profiling = s->profiling;
    s->profiling = true;
    pg_step_args st = *a;
    int rc = PG_OK;
    auto run = [&](int n, double *ms) -> int {
        collect_stages(s);
        for (auto &v : s->stage_ms) v = 0.0;
        for (int i = 0; i < n; ++i) {
            int r = pg_step(s, &st, objects, n_objects, nullptr);
            if (r) return r;
            st.first_step = 0;
            st.step += 1;
        }
        collect_stages(s);
        if (ms) *ms = pass_ms(s) / n;
        return PG_OK;
    };
    // block size x blocks per SM x deposit aggregation (mixed form)
    pg_tuning best{};
    double best_ms = 1e300;
    const int threads[] = {128, 256, 512};
    const int bps[] = {2, 4, 8, 16};
    const int saved_interval = s->cfg.sort_interval;
    s->cfg.sort_interval = 1 << 30;   // no sorts while timing the launch configurations
    if ((rc = do_sort(s))) goto done;
    if ((rc = run(1, nullptr))) goto done;
    for (int th : threads)
        for (int b : bps)
            for (int agg = 0; agg <= (is_mixed(s) ? 1 : 0); ++agg) {
                pg_tuning t{th, b, agg, 0, 0.0, 0.0};
                if ((rc = pg_set_tuning(s, &t))) goto done;
                if ((rc = do_sort(s))) goto done;
                double ms = 0;
                if ((rc = run(k, &ms))) goto done;
                if (ms < best_ms) { best_ms = ms; best = t; }
            }
    if ((rc = pg_set_tuning(s, &best))) goto done;
    {
        // sort interval: the sort's cost against the growth of the pass time
        // with the steps since the last sort
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, s->stream);
        rc = do_sort(s);
        cudaEventRecord(e1, s->stream);
        cudaEventSynchronize(e1);
        float sort_ms = 0;
        cudaEventElapsedTime(&sort_ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc) goto done;
        const int horizon = 40;
        std::vector<double> t(horizon, 0.0);
        for (int i = 0; i < horizon; ++i)
            if ((rc = run(1, &t[i]))) goto done;
        double best_cost = 1e300;
        int best_i = saved_interval;
        for (int I : {5, 10, 20, 40}) {
            double mean = 0.0;
            for (int i = 0; i < I; ++i) mean += t[i] - t[0];
            const double cost = sort_ms / I + mean / I;
            if (cost < best_cost) { best_cost = cost; best_i = I; }
        }
        best.sort_interval = best_i;
        best.pass_ms = best_ms;
        best.sort_ms = sort_ms;
    }
done:
    s->cfg.sort_interval = best.sort_interval > 0 ? best.sort_interval : saved_interval;
    s->profiling = profiling;
    if (rc) return rc;
    if (out) *out = best;
    return do_sort(s);
}

// Device time of a named stage over the steps since the last reset.
static double stage_ms_named(pg_sim *s, const char *name) {
    for (size_t k = 0; k < s->stage_names.size(); ++k)
        if (s->stage_names[k] == name) return s->stage_ms[k];
    return 0.0;
}

int pg_amg_set_strength(pg_sim *s, double theta) {
    if (!s) return fail(PG_ERR_ARG, "pg_amg_set_strength: NULL handle");
    if (!(theta >= 0.0 && theta < 1.0)) return fail(PG_ERR_ARG, "pg_amg_set_strength: theta must lie in [0, 1)");
    if (s->amg_A0.n == 0) return fail(PG_ERR_ARG, "pg_amg_set_strength: the solver has no AMG preconditioner");
    if (theta == s->amg_theta && s->use_amg) return PG_OK;
    PG_CUDA(cudaStreamSynchronize(s->stream));
    drop_graphs(s);
    const double old = s->amg_theta;
    s->amg_theta = theta;
    int rc = rebuild_amg(s);
    if (rc) {
        // keep the handle usable: back to the previous hierarchy
        const std::string msg = pg_last_error();
        s->amg_theta = old;
        if (rebuild_amg(s) == PG_OK) return fail(rc, msg);
    }
    return rc;
}

int pg_amg_get_strength(pg_sim *s, double *theta) {
    if (!s || !theta) return fail(PG_ERR_ARG, "pg_amg_get_strength: NULL argument");
    *theta = s->amg_theta;
    return PG_OK;
}

int pg_autotune_amg(pg_sim *s, const pg_step_args *a, pg_object *objects, int32_t n_objects, int32_t steps_per_trial,
                    const double *thetas, int32_t n_thetas, double *best_theta, double *best_ms) {
    if (!s || !a) return fail(PG_ERR_ARG, "pg_autotune_amg: NULL argument");
    if (n_thetas < 0 || (n_thetas > 0 && !thetas)) return fail(PG_ERR_ARG, "pg_autotune_amg: bad candidates");
    if (s->amg_A0.n == 0) return fail(PG_ERR_ARG, "pg_autotune_amg: the solver has no AMG preconditioner");
    static const double kDefault[] = {0.0, 0.01, 0.02};
    const double *cand = n_thetas > 0 ? thetas : kDefault;
    const int nc = n_thetas > 0 ? n_thetas : 3;
    const int k = std::max(1, steps_per_trial);
    const bool profiling = s->profiling;
    s->profiling = true;
    pg_step_args st = *a;
    int rc = PG_OK;
    const double theta0 = s->amg_theta;
    double bt = theta0, bms = 1e300;
    for (int c = 0; c < nc && rc == PG_OK; ++c) {
        if ((rc = pg_amg_set_strength(s, cand[c]))) break;
        collect_stages(s);
        for (auto &v : s->stage_ms) v = 0.0;
        for (int i = 0; i < k && rc == PG_OK; ++i) {
            rc = pg_step(s, &st, objects, n_objects, nullptr);
            st.first_step = 0;
            st.step += 1;
        }
        if (rc) break;
        collect_stages(s);
        const double ms = stage_ms_named(s, "pcg") / k;
        if (ms < bms) { bms = ms; bt = cand[c]; }
    }
    s->profiling = profiling;
    if (rc) {
        // back to the threshold the call started with
        const std::string msg = pg_last_error();
        if (pg_amg_set_strength(s, theta0) == PG_OK) return fail(rc, msg);
        return rc;
    }
    if ((rc = pg_amg_set_strength(s, bt))) return rc;
    if (best_theta) *best_theta = bt;
    if (best_ms) *best_ms = bms;
    return PG_OK;
}

// ---- adjoint of K fused steps (FP64 form) ---------------------------------

static void adj_free(pg_sim *s) {
    for (void *p : s->adj.mem) cudaFree(p);
    s->adj = pg_sim::Adjoint{};
}

static int adj_alloc(pg_sim *s, void **p, size_t bytes) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(8, bytes));
    if (e != cudaSuccess) return fail(PG_ERR_CUDA, std::string("adjoint cudaMalloc: ") + cudaGetErrorString(e));
    s->adj.mem.push_back(q);
    *p = q;
    return PG_OK;
}

// copy the particle state (positions, velocities, cells) of the current buffer
static int adj_save(pg_sim *s, double *x, int32_t *c) {
    const DevParticles &P = s->P[s->cur];
    const size_t n = (size_t)s->adj.n;
    double *src[6] = {P.x, P.y, P.z, P.vx, P.vy, P.vz};
    for (int k = 0; k < 6; ++k)
        PG_CUDA(cudaMemcpyAsync(x + k * n, src[k], sizeof(double) * n, cudaMemcpyDeviceToDevice, s->stream));
    PG_CUDA(cudaMemcpyAsync(c, P.cell, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s->stream));
    return PG_OK;
}

static int adj_restore(pg_sim *s, const double *x, const int32_t *c) {
    const DevParticles &P = s->P[s->cur];
    const size_t n = (size_t)s->adj.n;
    double *dst[6] = {P.x, P.y, P.z, P.vx, P.vy, P.vz};
    for (int k = 0; k < 6; ++k)
        PG_CUDA(cudaMemcpyAsync(dst[k], x + k * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, s->stream));
    PG_CUDA(cudaMemcpyAsync(P.cell, c, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s->stream));
    s->rho_valid = false;
    return PG_OK;
}

static pg_step_args adj_step_args(const pg_sim *s, int step) {
    pg_step_args a = s->adj.args;
    a.first_step = (step == 0 && s->adj.args.first_step) ? 1 : 0;
    a.step = s->adj.args.step + (uint64_t)step;
    a.inject = 0;
    return a;
}

int pg_adjoint_forward(pg_sim *s, const pg_step_args *a, pg_object *objects, int32_t n_objects, int32_t n_steps,
                       int32_t ckpt_every, const double *rho_target, double *loss) {
    if (!s || !a || !rho_target || n_steps < 1 || ckpt_every < 1 || (n_objects > 0 && !objects))
        return fail(PG_ERR_ARG, "pg_adjoint_forward: bad arguments");
    if (is_mixed(s)) return fail(PG_ERR_ARG, "pg_adjoint_forward: the adjoint runs in the FP64 form");
    if (a->inject || a->efield_cg1 || a->B[0] != 0.0 || a->B[1] != 0.0 || a->B[2] != 0.0)
        return fail(PG_ERR_ARG, "pg_adjoint_forward: push with the DG0 field and B = 0, no injection");
    if (s->circuit_ready) return fail(PG_ERR_ARG, "pg_adjoint_forward: objects at fixed potentials only");
    if (s->adj.ready) { s->cfg.sort_interval = s->adj.saved_sort_interval; }
    adj_free(s);
    auto &J = s->adj;
    J.K = n_steps;
    J.C = ckpt_every;
    J.args = *a;
    J.objects.assign(objects, objects + n_objects);
    J.saved_sort_interval = s->cfg.sort_interval;
    int rc = do_sort(s);            // compact the slots once; no sort during the K steps
    if (rc) return rc;
    s->cfg.sort_interval = 1 << 30;
    J.n = s->n_slots;
    const size_t n = (size_t)J.n, nd = (size_t)s->ndof;
    const int nck = (n_steps + ckpt_every - 1) / ckpt_every;
    J.ck_x.resize(nck);
    J.ck_c.resize(nck);
    for (int k = 0; k < nck; ++k)
        if ((rc = adj_alloc(s, (void **)&J.ck_x[k], sizeof(double) * 6 * n)) ||
            (rc = adj_alloc(s, (void **)&J.ck_c[k], sizeof(int32_t) * n)))
            return rc;
    if ((rc = adj_alloc(s, (void **)&J.fin_x, sizeof(double) * 6 * n)) ||
        (rc = adj_alloc(s, (void **)&J.fin_c, sizeof(int32_t) * n)) ||
        (rc = adj_alloc(s, (void **)&J.rec_c, sizeof(int32_t) * (size_t)ckpt_every * n)) ||
        (rc = adj_alloc(s, (void **)&J.bar, sizeof(double) * 6 * n)) ||
        (rc = adj_alloc(s, (void **)&J.Ebar, sizeof(double) * 3 * (size_t)s->nc)) ||
        (rc = adj_alloc(s, (void **)&J.phibar, sizeof(double) * nd)) ||
        (rc = adj_alloc(s, (void **)&J.y, sizeof(double) * nd)) ||
        (rc = adj_alloc(s, (void **)&J.rhobar, sizeof(double) * nd)) ||
        (rc = adj_alloc(s, (void **)&J.target, sizeof(double) * nd)) ||
        (rc = adj_alloc(s, (void **)&J.small, sizeof(double) * 16)))
        return rc;
    PG_CUDA(cudaMemcpyAsync(J.target, rho_target, sizeof(double) * nd, cudaMemcpyHostToDevice, s->stream));
    if (s->n_obj > 0) {
        // dphi/dV_k: the unit-potential Laplace solutions (the circuit's when
        // it has them, else solved here; the charge is re-deposited by the
        // first step)
        if ((rc = adj_alloc(s, (void **)&J.lap, sizeof(double) * nd * (size_t)s->n_obj)) ||
            (rc = adj_alloc(s, (void **)&J.gpot, sizeof(double) * (size_t)s->n_obj)))
            return rc;
        for (int k = 0; k < s->n_obj; ++k) {
            if (s->lap) {
                PG_CUDA(cudaMemcpyAsync(J.lap + (size_t)k * nd, s->lap + (size_t)k * nd, sizeof(double) * nd,
                                        cudaMemcpyDeviceToDevice, s->stream));
                continue;
            }
            std::vector<double> pot(s->n_obj, 0.0);
            pot[k] = 1.0;
            if ((rc = poisson_solve_internal(s, pot.data(), true, false, std::min(1e-13, s->cfg.pcg_rtol),
                                             std::min(1e-15, s->cfg.pcg_atol), nullptr)))
                return rc;
            PG_CUDA(cudaMemcpyAsync(J.lap + (size_t)k * nd, s->phi, sizeof(double) * nd, cudaMemcpyDeviceToDevice,
                                    s->stream));
        }
        s->phi_valid = false;
    }
    int64_t live0 = 0, neg = 0, pos = 0;
    if ((rc = pg_num_particles(s, &live0, &neg, &pos))) return rc;
    std::vector<pg_object> obj = J.objects;
    for (int k = 0; k < n_steps; ++k) {
        if (k % ckpt_every == 0 && (rc = adj_save(s, J.ck_x[k / ckpt_every], J.ck_c[k / ckpt_every]))) return rc;
        const pg_step_args ak = adj_step_args(s, k);
        if ((rc = pg_step(s, &ak, obj.data(), (int32_t)obj.size(), nullptr))) return rc;
    }
    int64_t live1 = 0;
    if ((rc = pg_num_particles(s, &live1, &neg, &pos))) return rc;
    if (live1 != live0 || s->n_slots != J.n)
        return fail(PG_ERR_ARG, "pg_adjoint_forward: particles were absorbed or added during the steps");
    // rho_K and the loss ||rho_K - target||^2
    rho_from_acc(s);
    PG_CUDA(cudaMemsetAsync(J.small, 0, sizeof(double) * 16, s->stream));
    launch_loss_grad(s->ndof, s->rho, J.target, J.rhobar, J.small + 3, s->stream);
    if ((rc = adj_save(s, J.fin_x, J.fin_c))) return rc;
    double l = 0;
    PG_CUDA(cudaMemcpyAsync(&l, J.small + 3, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    if (loss) *loss = l;
    J.ready = true;
    return PG_OK;
}

// rhobar = M P A^+ P phibar (Dirichlet rows of phibar zeroed)
static int adj_poisson(pg_sim *s) {
    auto &J = s->adj;
    if (s->has_dirichlet) launch_zero_dirichlet(s->ndof, s->bc_kind, J.phibar, s->stream);
    PG_CUDA(cudaMemsetAsync(J.y, 0, sizeof(double) * s->ndof, s->stream));
    PcgArgs a{};
    a.n = s->ndof;
    a.slice_ptr = s->A_sptr; a.slice_width = s->A_swidth; a.col = s->A_col; a.val = s->A_val; a.dinv = s->A_dinv;
    a.b = J.phibar; a.x = J.y; a.r = s->r; a.z = s->z; a.p0 = s->p0; a.p1 = s->p1; a.Ap = s->Ap;
    a.partials = s->pcg_part;
    a.rtol = 1e-13; a.atol = 0.0;
    a.max_iter = std::max(s->cfg.pcg_max_iter, 4000);
    a.remove_mean = s->cfg.periodic ? 1 : 0;
    a.out_iter = s->pcg_out_i; a.out_status = s->pcg_out_i + 1;
    a.out_rr = s->pcg_out_d; a.out_bb = s->pcg_out_d + 1;
    a.val32 = s->A_val32; a.dinv32 = s->A_dinv32;
    a.r32 = s->r32; a.z32 = s->z32; a.p32 = s->p32; a.Ap32 = s->Ap32;
    const int e = s->use_amg ? launch_pcg_amg(a, s->amg, s->stream) : launch_pcg(a, s->stream);
    if (e) return fail(PG_ERR_CUDA, std::string("adjoint PCG launch: ") + cudaGetErrorString((cudaError_t)e));
    launch_csr_matvec(s->ndof, s->M_row, s->M_col, s->M_val, J.y, J.rhobar, s->stream);
    return PG_OK;
}

int pg_adjoint_backward(pg_sim *s, double *grad_v, int64_t n_out, double *grad_E0, double *grad_x0) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    auto &J = s->adj;
    if (!J.ready) return fail(PG_ERR_STATE, "pg_adjoint_backward: call pg_adjoint_forward first");
    const size_t n = (size_t)J.n;
    double *xb = J.bar, *yb = J.bar + n, *zb = J.bar + 2 * n, *vxb = J.bar + 3 * n, *vyb = J.bar + 4 * n,
           *vzb = J.bar + 5 * n;
    const DevParticles &P = s->P[s->cur];
    PG_CUDA(cudaMemsetAsync(J.bar, 0, sizeof(double) * 6 * n, s->stream));
    PG_CUDA(cudaMemsetAsync(J.small, 0, sizeof(double) * 3, s->stream));
    if (J.gpot) PG_CUDA(cudaMemsetAsync(J.gpot, 0, sizeof(double) * (size_t)s->n_obj, s->stream));
    // d loss / d x_K through rho_K (cells at step K); rhobar holds 2 (rho_K - target)
    launch_adj_deposit(s->dm, J.n, J.fin_c, P.sp, s->d_q, J.rhobar, xb, yb, zb, s->stream);
    std::vector<pg_object> obj = J.objects;
    int rc = PG_OK;
    const int nck = (int)J.ck_x.size();
    for (int seg = nck - 1; seg >= 0 && rc == PG_OK; --seg) {
        const int k0 = seg * J.C, k1 = std::min(J.K, k0 + J.C);
        // recompute the segment, recording the cells at the start of each step
        if ((rc = adj_restore(s, J.ck_x[seg], J.ck_c[seg]))) break;
        for (int k = k0; k < k1 && rc == PG_OK; ++k) {
            PG_CUDA(cudaMemcpyAsync(J.rec_c + (size_t)(k - k0) * n, s->P[s->cur].cell, sizeof(int32_t) * n,
                                    cudaMemcpyDeviceToDevice, s->stream));
            const pg_step_args ak = adj_step_args(s, k);
            rc = pg_step(s, &ak, obj.data(), (int32_t)obj.size(), nullptr);
        }
        if (rc) break;
        for (int k = k1 - 1; k >= k0 && rc == PG_OK; --k) {
            const pg_step_args ak = adj_step_args(s, k);
            const double dt_push = ak.first_step ? 0.5 * ak.dt : ak.dt;
            double coef[kMaxSpecies] = {0};
            for (int sp = 0; sp < s->n_species; ++sp) coef[sp] = dt_push * (s->q[sp] / s->m[sp]);
            PG_CUDA(cudaMemcpyAsync(J.small + 8, coef, sizeof(coef), cudaMemcpyHostToDevice, s->stream));
            const int32_t *cells = J.rec_c + (size_t)(k - k0) * n;
            PG_CUDA(cudaMemsetAsync(J.Ebar, 0, sizeof(double) * 3 * (size_t)s->nc, s->stream));
            PG_CUDA(cudaMemsetAsync(J.phibar, 0, sizeof(double) * s->ndof, s->stream));
            launch_adj_move_push(J.n, cells, P.sp, J.small + 8, ak.dt, xb, yb, zb, vxb, vyb, vzb, J.Ebar, J.small,
                                 s->stream);
            launch_adj_field(s->dm, J.Ebar, J.phibar, s->stream);
            for (int o = 0; o < s->n_obj && J.gpot; ++o)
                launch_dot_accum(s->ndof, J.phibar, J.lap + (size_t)o * s->ndof, J.gpot + o, s->stream);
            if ((rc = adj_poisson(s))) break;
            launch_adj_deposit(s->dm, J.n, cells, P.sp, s->d_q, J.rhobar, xb, yb, zb, s->stream);
        }
    }
    if (rc == PG_OK) {
        if (grad_v || grad_x0) {
            double *out = nullptr;
            PG_CUDA(cudaMalloc(&out, sizeof(double) * 3 * std::max<int64_t>(1, n_out)));
            cudaError_t e = cudaSuccess;
            if (grad_v) {
                cudaMemsetAsync(out, 0, sizeof(double) * 3 * n_out, s->stream);
                launch_scatter_by_id(J.n, J.ck_c[0], P.pid, 0, n_out, vxb, vyb, vzb, out, s->stream);
                e = cudaMemcpyAsync(grad_v, out, sizeof(double) * 3 * n_out, cudaMemcpyDeviceToHost, s->stream);
            }
            if (grad_x0 && e == cudaSuccess) {
                cudaStreamSynchronize(s->stream);
                cudaMemsetAsync(out, 0, sizeof(double) * 3 * n_out, s->stream);
                launch_scatter_by_id(J.n, J.ck_c[0], P.pid, 0, n_out, xb, yb, zb, out, s->stream);
                e = cudaMemcpyAsync(grad_x0, out, sizeof(double) * 3 * n_out, cudaMemcpyDeviceToHost, s->stream);
            }
            cudaStreamSynchronize(s->stream);
            cudaFree(out);
            if (e != cudaSuccess) rc = fail(PG_ERR_CUDA, cudaGetErrorString(e));
        }
        if (grad_E0) {
            double g[3];
            cudaMemcpyAsync(g, J.small, sizeof(g), cudaMemcpyDeviceToHost, s->stream);
            cudaStreamSynchronize(s->stream);
            for (int j = 0; j < 3; ++j) grad_E0[j] = g[j];
        }
    }
    // back to the state after the K steps
    int rc2 = adj_restore(s, J.fin_x, J.fin_c);
    PG_CUDA(cudaStreamSynchronize(s->stream));
    if (rc == PG_OK) rc = rc2;
    if (rc == PG_OK) rc = check_state(s);
    return rc;
}

int pg_adjoint_potential_gradient(pg_sim *s, double *grad_pot, int32_t n_objects) {
    if (!s || (n_objects > 0 && !grad_pot)) return fail(PG_ERR_ARG, "pg_adjoint_potential_gradient: bad arguments");
    if (!s->adj.ready) return fail(PG_ERR_STATE, "pg_adjoint_potential_gradient: call pg_adjoint_forward first");
    if (n_objects != s->n_obj) return fail(PG_ERR_ARG, "pg_adjoint_potential_gradient: n_objects differs from the mesh's");
    if (n_objects == 0) return PG_OK;
    PG_CUDA(cudaMemcpyAsync(grad_pot, s->adj.gpot, sizeof(double) * (size_t)n_objects, cudaMemcpyDeviceToHost,
                            s->stream));
    PG_CUDA(cudaStreamSynchronize(s->stream));
    return PG_OK;
}

int pg_adjoint_release(pg_sim *s) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    if (s->adj.ready) s->cfg.sort_interval = s->adj.saved_sort_interval;
    adj_free(s);
    return PG_OK;
}

int pg_step(pg_sim *s, const pg_step_args *a, pg_object *objects, int32_t n_objects, pg_step_result *res) {
    if (!s || !a || (n_objects > 0 && !objects)) return fail(PG_ERR_ARG, "pg_step: bad arguments");
    pg_step_result out{};
    int rc;
    // distribute
    {
        StageScope t(s, "distributor");
        if (!s->rho_valid) {
            rc = deposit_into_acc(s);
            if (rc) return rc;
        }
        rho_from_acc(s);
    }
    // poisson (+ circuit)
    {
        StageScope t(s, "poisson");
        pg_solve_info info{};
        if (s->circuit_ready) {
            rc = solve_circuit_internal(s, objects, n_objects, &info);
        } else {
            std::vector<double> pot(std::max(1, s->n_obj), 0.0);
            for (int k = 0; k < n_objects; ++k) {
                const int i = object_index(s, objects[k].bnd_id);
                if (i >= 0) pot[i] = objects[k].potential;
            }
            rc = poisson_solve_internal(s, pot.data(), false, true, s->cfg.pcg_rtol, s->cfg.pcg_atol, &info);
        }
        out.pcg_iterations = info.iterations;
        out.pcg_residual = info.residual;
        if (rc) return rc;
    }
    if (a->efield_cg1) {
        rc = esolver_internal(s, a->E0, nullptr);
        if (rc) return rc;
    } else if (!is_mixed(s)) {
        StageScope t(s, "efield");
        step_field_f64(s, a->E0);
    }
    if (a->potential_energy) {
        // particle_potential_energy_cg1 at the time loop's place: particles at
        // the step's start, the step's potential (interaction.cpp:367-372)
        StageScope t(s, "PE");
        if ((rc = diag_scratch(s))) return rc;
        launch_potential_energy(s->dm, s->P[s->cur], s->n_slots, is_mixed(s), s->d_q, s->phi, s->diag_acc, s->stream);
        PG_CUDA(cudaMemcpyAsync(&out.PE, s->diag_acc, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    }
    // accelerator + move + update, depositing the next step's charge
    {
        StageScope t(s, "push_move_update_deposit");
        const double dt_push = a->first_step ? 0.5 * a->dt : a->dt;
        PushParams pp;
        fill_push(s, pp, dt_push, a->B, a->use_accel != 0);
        pp.cg1 = a->efield_cg1 ? 1 : 0;
        MoveParams mp{};
        mp.dt = a->dt;
        mp.periodic = a->periodic_move;
        for (int j = 0; j < 3; ++j) mp.Ld[j] = a->Ld[j];
        PG_CUDA(cudaMemsetAsync(s->state->absorbed, 0, sizeof(s->state->absorbed), s->stream));
        if (is_mixed(s)) {
            PG_CUDA(cudaMemsetAsync(s->rho_fixed, 0, sizeof(unsigned long long) * s->ndof, s->stream));
            MixedParams xp;
            fill_mixed(s, xp, dt_push, a->B, a->use_accel != 0, a->dt, a->periodic_move != 0, a->Ld);
            xp.cg1 = a->efield_cg1 ? 1 : 0;
            if (!a->efield_cg1) pass_field(s, xp, a->E0);
            if (s->n_slots > 0)
                launch_mixed_pass(s->dm, s->P[s->cur], s->n_slots, xp, true, true, true, true, s->cfg.max_walk_steps,
                                  s->rho_fixed, s->state, s->partials, s->n_part, s->ke_dev, s->stream);
        } else {
            PG_CUDA(cudaMemsetAsync(s->rho_acc, 0, sizeof(double) * s->ndof, s->stream));
        }
        if (s->n_slots > 0 && !is_mixed(s))
            launch_fused_step(s->dm, s->P[s->cur], s->n_slots, pp, mp, s->cfg.max_walk_steps, s->d_q, s->rho_acc,
                              s->state, s->partials, s->n_part, s->ke_dev, s->stream);
        else if (s->n_slots == 0)
            PG_CUDA(cudaMemsetAsync(s->ke_dev, 0, sizeof(double), s->stream));
        double ke = 0;
        PG_CUDA(cudaMemcpyAsync(&ke, s->ke_dev, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        rc = check_state(s);
        if (rc) return rc;
        out.KE = ke;
        absorbed_to_objects(s, objects, n_objects, a->dt, &out.n_absorbed);
    }
    if (a->inject) {
        StageScope t(s, "injector");
        rc = inject_internal(s, a->dt, a->seed, a->step, true, &out.n_injected);
        if (rc) return rc;
    }
    s->rho_valid = true;
    ++s->step_count;
    if (s->step_count % s->cfg.sort_interval == 0) {
        StageScope t(s, "sort");
        rc = do_sort(s);
        if (rc) return rc;
    }
    collect_stages(s);
    int64_t tot = 0;
    for (int k = 0; k < s->n_species; ++k) tot += s->state_h->live[k];
    out.n_particles = tot;
    if (res) *res = out;
    return PG_OK;
}

int pg_event_record(pg_sim *s, int32_t slot) {
    if (!s || slot < 0 || slot >= 16) return fail(PG_ERR_ARG, "pg_event_record: bad slot");
    if (!s->user_ev[slot]) PG_CUDA(cudaEventCreate(&s->user_ev[slot]));
    PG_CUDA(cudaEventRecord(s->user_ev[slot], s->stream));
    return PG_OK;
}

int pg_event_elapsed(pg_sim *s, int32_t a, int32_t b, double *ms) {
    if (!s || !ms || a < 0 || b < 0 || a >= 16 || b >= 16 || !s->user_ev[a] || !s->user_ev[b])
        return fail(PG_ERR_ARG, "pg_event_elapsed: slot not recorded");
    PG_CUDA(cudaEventSynchronize(s->user_ev[b]));
    float f = 0;
    PG_CUDA(cudaEventElapsedTime(&f, s->user_ev[a], s->user_ev[b]));
    *ms = f;
    return PG_OK;
}

int pg_poisson_layout_get(pg_sim *s, pg_poisson_layout *out) {
    if (!s || !out) return fail(PG_ERR_ARG, "pg_poisson_layout_get: null argument");
    *out = pg_poisson_layout{};
    out->n_rows = s->ndof;
    out->nnz = s->a_nnz;
    out->sell_entries = s->a_sell;
    out->precond = s->cfg.pcg_precond;
    out->levels = s->use_amg ? s->amg.nlev : 0;
    for (int l = 0; l < out->levels && l < PG_MAX_AMG_LEVELS; ++l) {
        out->level_rows[l] = s->amg_rows[l];
        out->level_nnz[l] = s->amg_nnz[l];
        out->level_nnz_p[l] = s->amg_nnz_p[l];
    }
    out->cycle_nnz_g = s->use_amg ? s->amg_nnz_g : 0;
    out->cycle_nnz_u1 = s->use_amg ? s->amg_nnz_u1 : 0;
    out->cycle_bytes = s->use_amg ? s->amg_cycle_bytes : 0;
    return PG_OK;
}

int pg_launch_count(int64_t *n) {
    if (!n) return fail(PG_ERR_ARG, "pg_launch_count: NULL argument");
    *n = launches_so_far();
    return PG_OK;
}

int pg_synchronize(pg_sim *s) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    PG_CUDA(cudaStreamSynchronize(s->stream));
    if (s->copy_stream) {
        PG_CUDA(cudaStreamSynchronize(s->copy_stream));
        s->phi_copy_pending = false;
    }
    return PG_OK;
}

const char *pg_stage_name(pg_sim *s, int32_t index) {
    if (!s || index < 0 || index >= (int32_t)s->stage_names.size()) return nullptr;
    return s->stage_names[index].c_str();
}

int pg_set_profiling(pg_sim *s, int32_t on) {
    if (!s) return fail(PG_ERR_ARG, "NULL handle");
    s->profiling = on != 0;
    return PG_OK;
}

int pg_stage_times(pg_sim *s, double *ms, int32_t capacity, int32_t *n_stages) {
    if (!s || !n_stages) return fail(PG_ERR_ARG, "pg_stage_times: NULL argument");
    collect_stages(s);
    *n_stages = (int32_t)s->stage_names.size();
    for (int32_t k = 0; k < *n_stages && k < capacity; ++k) {
        if (ms) ms[k] = s->stage_ms[k];
        s->stage_ms[k] = 0.0;
    }
    return PG_OK;
}

}  // extern "C"
