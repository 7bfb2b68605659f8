// Per-step bookkeeping on the device, so that a whole time step runs without
// host round trips and can be captured as a CUDA graph:
//   object currents and charges from the absorbed counts (Population::update's
//   current bookkeeping, punc/include/punc/population.h:686-698),
//   CircuitCM pre_solve / post_solve (punc/src/object_CM.cpp:53-60, 275-357)
//   in the engine's host loop order (single thread, FP64, no contraction: the
//   same bits as the host path),
//   the superposition phi = phi0 + sum V_k L_k with device potentials,
//   particle and RNG counters, and one row of step results.
#include <cuda_runtime.h>

#include "pg_device.cuh"

namespace pg {

namespace {

// counts: [0] slots in use, [1] next particle id, [2] RNG step, [3] result row
__global__ void k_inject_commit(int64_t *counts, const DevState *st) {
    const int64_t t = st->inject_total;
    counts[0] += t;
    counts[1] += t;
}

// Object bookkeeping after update (population.h:686-698): current = sum of the
// absorbed charge; charge += current; current /= dt.
__global__ void k_objects_update(const DevState *st, const double *q, int n_species, const int64_t *tags, int n_obj,
                                 double *obj, double dt) {
    for (int k = 0; k < n_obj; ++k) {
        const int64_t tag = tags[k];
        double cur = 0.0;
        if (tag > 0 && tag < kMaxTags)
            for (int sp = 0; sp < n_species; ++sp) cur += (double)st->absorbed[tag][sp] * q[sp];
        obj[4 * k + 1] = cur;
    }
    for (int k = 0; k < n_obj; ++k) {
        obj[4 * k + 0] += obj[4 * k + 1];
        obj[4 * k + 1] /= dt;
    }
}

// CircuitCM::pre_solve (object_CM.cpp:53-60): current sources move charge;
// potentials to zero.  isrc: [n][3] (node_a, node_b, value).
__global__ void k_circuit_pre(const double *isrc, int n_isrc, double circ_dt, int n_obj, double *obj,
                              double *obj_pot) {
    for (int k = 0; k < n_isrc; ++k) {
        const int a = (int)isrc[3 * k], b = (int)isrc[3 * k + 1];
        const double dQ = isrc[3 * k + 2] * circ_dt;
        if (a != -1) obj[4 * a + 0] -= dQ;
        if (b != -1) obj[4 * b + 0] += dQ;
    }
    for (int i = 0; i < n_obj; ++i) { obj[4 * i + 2] = 0.0; obj_pot[i] = 0.0; }
}

// CircuitCM::post_solve (object_CM.cpp:275-357) with the image charges img:
// circuit vector from the charge-sharing groups and the fixed-voltage sets,
// then potentials and charges from the inverse circuit matrix.
__global__ void k_circuit_post(const CircuitDev c, const double *img, double *obj, double *obj_pot) {
    const int n = c.n;
    double *cv = c.cv;
    for (int g = 0; g < c.n_groups; ++g) {
        double col = 0.0;
        for (int k = c.g_ptr[g]; k < c.g_ptr[g + 1]; ++k) col += obj[4 * c.g_mem[k] + 0];
        cv[n + c.g_mem[c.g_ptr[g]]] = col;
    }
    for (int g = 0; g < c.n_groups; ++g) {
        const int g0 = c.g_mem[c.g_ptr[g]];
        double col = 0.0;
        for (int k = c.g_ptr[g]; k < c.g_ptr[g + 1]; ++k) col += c.inv_cap[g0 * n + c.g_mem[k]] * img[c.g_mem[k]];
        cv[g0] = col;
        for (int j = c.g_ptr[g] + 1; j < c.g_ptr[g + 1]; ++j) {
            const int gj = c.g_mem[j];
            col = 0.0;
            for (int k = c.g_ptr[g]; k < c.g_ptr[g + 1]; ++k) col += c.inv_cap[gj * n + c.g_mem[k]] * img[c.g_mem[k]];
            cv[n + gj] = col;
        }
    }
    for (int f = 0; f < c.n_fv; ++f)
        for (int j = c.f_ptr[f]; j < c.f_ptr[f + 1]; ++j) {
            const int fj = c.f_mem[j];
            double col = 0.0;
            for (int k = c.f_ptr[f]; k < c.f_ptr[f + 1]; ++k) col += c.inv_cap[fj * n + c.f_mem[k]] * img[c.f_mem[k]];
            cv[n + fj] = col;
        }
    for (int i = 0; i < n; ++i) {
        double p = 0.0, ch = 0.0;
        for (int j = 0; j < 2 * n; ++j) p += c.inv_circ[i * 2 * n + j] * cv[j];
        for (int j = 0; j < 2 * n; ++j) ch += c.inv_circ[(n + i) * 2 * n + j] * cv[j];
        obj[4 * i + 2] = p;
        obj[4 * i + 0] = ch;
        obj_pot[i] = p;
    }
}

__global__ void k_superpose_dev(const double *__restrict__ phi0, const double *__restrict__ lap,
                                const double *__restrict__ pot, const int32_t *__restrict__ rng, int n_obj, int32_t n,
                                double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = phi0[i];
    for (int k = 0; k < n_obj; ++k)
        if (!rng || (i >= rng[2 * k] && i < rng[2 * k + 1])) v = v + pot[k] * lap[(size_t)k * n + i];
    out[i] = v;
}

// One result row: KE, live particles, absorbed, injected (kept), PCG
// iterations, ||r||, then per object current, charge, potential.  One warp:
// lanes sum the per-tag absorbed counts, lane 0 writes the row.
__global__ void k_step_record(double *rows, int row_len, int64_t *counts, const double *ke, const DevState *st,
                              int n_species, const int32_t *pcg_i, const double *pcg_d, const double *obj, int n_obj) {
    const int lane = threadIdx.x;
    int64_t absorbed = 0;
    for (int t = lane; t < kMaxTags; t += 32)
        for (int k = 0; k < n_species; ++k) absorbed += st->absorbed[t][k];
    for (int o = 16; o > 0; o >>= 1) absorbed += __shfl_down_sync(0xffffffffu, absorbed, o);
    if (lane != 0) return;
    double *r = rows + (size_t)counts[3] * row_len;
    int64_t live = 0, injected = 0;
    for (int k = 0; k < n_species; ++k) live += st->live[k];
    for (int k = 0; k < kMaxSpecies; ++k) injected += st->injected[k];
    r[0] = *ke;
    r[1] = (double)live;
    r[2] = (double)absorbed;
    r[3] = (double)injected;
    r[4] = pcg_i ? (double)pcg_i[0] : 0.0;
    r[5] = pcg_d ? sqrt(pcg_d[0]) : 0.0;
    for (int k = 0; k < n_obj; ++k) {
        r[6 + 3 * k] = obj[4 * k + 1];
        r[7 + 3 * k] = obj[4 * k + 0];
        r[8 + 3 * k] = obj[4 * k + 2];
    }
    counts[2] += 1;
    counts[3] += 1;
}

__global__ void k_set_count(int64_t *counts, const int64_t *cursor, int32_t nc) { counts[0] = cursor[nc]; }

}  // namespace

void launch_inject_commit(int64_t *counts, const DevState *st, cudaStream_t s) {
    count_launches(1);
    k_inject_commit<<<1, 1, 0, s>>>(counts, st);
}
void launch_objects_update(const DevState *st, const double *q, int n_species, const int64_t *tags, int n_obj,
                           double *obj, double dt, cudaStream_t s) {
    if (n_obj <= 0) return;
    count_launches(1);
    k_objects_update<<<1, 1, 0, s>>>(st, q, n_species, tags, n_obj, obj, dt);
}
void launch_circuit_pre(const double *isrc, int n_isrc, double circ_dt, int n_obj, double *obj, double *obj_pot,
                        cudaStream_t s) {
    count_launches(1);
    k_circuit_pre<<<1, 1, 0, s>>>(isrc, n_isrc, circ_dt, n_obj, obj, obj_pot);
}
void launch_circuit_post(const CircuitDev &c, const double *img, double *obj, double *obj_pot, cudaStream_t s) {
    count_launches(1);
    k_circuit_post<<<1, 1, 0, s>>>(c, img, obj, obj_pot);
}
void launch_superpose_dev(const double *phi0, const double *lap, const double *pot, const int32_t *rng, int n_obj,
                         int32_t n, double *out, cudaStream_t s) {
    count_launches(1);
    k_superpose_dev<<<(n + 255) / 256, 256, 0, s>>>(phi0, lap, pot, rng, n_obj, n, out);
}
void launch_step_record(double *rows, int row_len, int64_t *counts, const double *ke, const DevState *st,
                        int n_species, const int32_t *pcg_i, const double *pcg_d, const double *obj, int n_obj,
                        cudaStream_t s) {
    count_launches(1);
    k_step_record<<<1, 32, 0, s>>>(rows, row_len, counts, ke, st, n_species, pcg_i, pcg_d, obj, n_obj);
}
void launch_set_count(int64_t *counts, const int64_t *cursor, int32_t nc, cudaStream_t s) {
    count_launches(1);
    k_set_count<<<1, 1, 0, s>>>(counts, cursor, nc);
}

}  // namespace pg
