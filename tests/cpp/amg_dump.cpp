// Host-only view of the AMG set-up (puncpp_gb300/csrc/amg.cpp) for the CPU
// tests: builds the hierarchy of a CSR matrix and copies its levels out.
#include <cstdint>
#include <cstring>

#include "pg_amg.h"

using pg::AmgHierarchy;
using pg::Csr;

extern "C" {

void *amgd_setup(int64_t n, const int64_t *rp, const int32_t *ci, const double *v, int nullspace, double theta,
                 double theta_factor, int64_t coarse_max, int *rc) {
    pg::AmgParams prm;
    if (theta >= 0.0) prm.theta = theta;
    if (theta_factor > 0.0) prm.theta_factor = theta_factor;
    if (coarse_max > 0) prm.coarse_max = coarse_max;
    Csr A;
    A.n = A.m = n;
    A.rp.assign(rp, rp + n + 1);
    A.ci.assign(ci, ci + rp[n]);
    A.v.assign(v, v + rp[n]);
    auto *h = new AmgHierarchy;
    *rc = pg::amg_setup(A, *h, nullspace != 0, prm);
    return h;
}

int amgd_levels(void *p) { return (int)static_cast<AmgHierarchy *>(p)->levels.size(); }

static const Csr &pick(void *p, int l, int which) {
    const auto &L = static_cast<AmgHierarchy *>(p)->levels[l];
    const Csr *ops[] = {&L.A, &L.P, &L.R, &L.S, &L.ST};
    return *ops[which];
}

// rows, columns, entries of operator `which` (0 A, 1 P, 2 R, 3 S, 4 S^T) of level l
void amgd_shape(void *p, int l, int which, int64_t out[3]) {
    const Csr &M = pick(p, l, which);
    out[0] = M.n;
    out[1] = M.m;
    out[2] = (int64_t)M.ci.size();
}

void amgd_copy(void *p, int l, int which, int64_t *rp, int32_t *ci, double *v) {
    const Csr &M = pick(p, l, which);
    std::memcpy(rp, M.rp.data(), sizeof(int64_t) * M.rp.size());
    std::memcpy(ci, M.ci.data(), sizeof(int32_t) * M.ci.size());
    std::memcpy(v, M.v.data(), sizeof(double) * M.v.size());
}

double amgd_omega(void *p, int l) { return static_cast<AmgHierarchy *>(p)->levels[l].omega; }

void amgd_coarse_inv(void *p, double *out) {
    const auto &c = static_cast<AmgHierarchy *>(p)->coarse_inv;
    std::memcpy(out, c.data(), sizeof(double) * c.size());
}

void amgd_free(void *p) { delete static_cast<AmgHierarchy *>(p); }

// the device cycle's operators: which 0 = G, 1 = U1
void *amgd_cycle(void *p) {
    auto *c = new pg::AmgCycle;
    pg::amg_cycle_operators(*static_cast<AmgHierarchy *>(p), *c);
    return c;
}
void amgd_cycle_shape(void *p, int which, int64_t out[3]) {
    const auto *c = static_cast<pg::AmgCycle *>(p);
    const Csr &M = which == 0 ? c->G : c->U1;
    out[0] = M.n;
    out[1] = M.m;
    out[2] = (int64_t)M.ci.size();
}
void amgd_cycle_copy(void *p, int which, int64_t *rp, int32_t *ci, double *v) {
    const auto *c = static_cast<pg::AmgCycle *>(p);
    const Csr &M = which == 0 ? c->G : c->U1;
    std::memcpy(rp, M.rp.data(), sizeof(int64_t) * M.rp.size());
    std::memcpy(ci, M.ci.data(), sizeof(int32_t) * M.ci.size());
    std::memcpy(v, M.v.data(), sizeof(double) * M.v.size());
}
int amgd_cycle_offsets(void *p, int64_t *out) {
    const auto *c = static_cast<pg::AmgCycle *>(p);
    std::memcpy(out, c->stack_off.data(), sizeof(int64_t) * c->stack_off.size());
    return (int)c->stack_off.size();
}
void amgd_cycle_free(void *p) { delete static_cast<pg::AmgCycle *>(p); }
}
