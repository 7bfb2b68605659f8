// Smoothed-aggregation algebraic multigrid set-up (host, once per mesh).
//
// The reference preconditions its Poisson solve with hypre's algebraic
// multigrid (punc/src/object_CM.cpp:208-219, punc/src/poisson.cpp:298-304);
// this is the engine's own AMG hierarchy for the PCG on the
// Dirichlet-eliminated P1 matrix:
//   * strength: |a_ij| > theta sqrt(a_ii a_jj) (theta = 0 by default: every
//     coupling of the P1 Laplacian counts);
//   * aggregation in three passes (Vanek, Mandel, Brezina 1996): a node whose
//     strong neighbours are all free seeds an aggregate with them; left-over
//     nodes join a neighbouring aggregate; the rest aggregate among themselves.
//     Rows without off-diagonal entries (eliminated Dirichlet rows) are left
//     out of the coarse spaces: the Jacobi smoother solves them exactly;
//   * tentative prolongator: the constant on each aggregate; smoothed
//     prolongator P = (I - omega D^-1 A) P0 with omega = 4 / (3 rho(D^-1 A)),
//     rho from a power iteration;
//   * Galerkin coarse operator A_c = P^T A P, recursively, until the coarse
//     space has at most AmgParams::coarse_max rows; the coarsest level is
//     inverted densely;
//   * for the device V-cycle, S = (I - omega D^-1 A) P and S^T: with one
//     Jacobi sweep from zero before and one after the coarse correction the
//     V-cycle is B = W + S B_c S^T, W = omega D^-1 (2 I - A omega D^-1).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <vector>

#include "pg_amg.h"

namespace pg {

namespace {

// C = A * B (Gustavson, dense accumulator per row).
Csr spgemm(const Csr &A, const Csr &B) {
    Csr C;
    C.n = A.n;
    C.m = B.m;
    C.rp.assign(A.n + 1, 0);
    std::vector<double> acc(B.m, 0.0);
    std::vector<int64_t> mark(B.m, -1);
    std::vector<int32_t> cols;
    for (int64_t i = 0; i < A.n; ++i) {
        cols.clear();
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            const int32_t j = A.ci[k];
            const double a = A.v[k];
            for (int64_t l = B.rp[j]; l < B.rp[j + 1]; ++l) {
                const int32_t c = B.ci[l];
                if (mark[c] != i) { mark[c] = i; acc[c] = 0.0; cols.push_back(c); }
                acc[c] += a * B.v[l];
            }
        }
        std::sort(cols.begin(), cols.end());
        for (int32_t c : cols) { C.ci.push_back(c); C.v.push_back(acc[c]); }
        C.rp[i + 1] = (int64_t)C.ci.size();
    }
    return C;
}

Csr transpose(const Csr &A) {
    Csr T;
    T.n = A.m;
    T.m = A.n;
    T.rp.assign(A.m + 1, 0);
    for (int32_t c : A.ci) T.rp[c + 1]++;
    for (int64_t i = 0; i < A.m; ++i) T.rp[i + 1] += T.rp[i];
    T.ci.resize(A.ci.size());
    T.v.resize(A.v.size());
    std::vector<int64_t> cur(T.rp.begin(), T.rp.end() - 1);
    for (int64_t i = 0; i < A.n; ++i)
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            const int64_t o = cur[A.ci[k]]++;
            T.ci[o] = (int32_t)i;
            T.v[o] = A.v[k];
        }
    return T;
}

std::vector<double> diagonal(const Csr &A) {
    std::vector<double> d(A.n, 0.0);
    for (int64_t i = 0; i < A.n; ++i)
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
            if (A.ci[k] == i) d[i] = A.v[k];
    return d;
}

// Aggregates of the strong-connection graph; -1 for rows left out.
int64_t aggregate(const Csr &A, const std::vector<double> &d, double theta, std::vector<int64_t> &agg) {
    const int64_t n = A.n;
    agg.assign(n, -2);   // -2 free, -1 excluded
    auto strong = [&](int64_t i, int64_t k) {
        const int64_t j = A.ci[k];
        return j != i && std::fabs(A.v[k]) > theta * std::sqrt(std::fabs(d[i] * d[j]));
    };
    for (int64_t i = 0; i < n; ++i) {
        bool any = false;
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) any |= strong(i, k);
        if (!any) agg[i] = -1;
    }
    int64_t na = 0;
    // pass 1: roots whose strong neighbourhood is entirely free
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] != -2) continue;
        bool ok = true;
        for (int64_t k = A.rp[i]; k < A.rp[i + 1] && ok; ++k)
            if (strong(i, k) && agg[A.ci[k]] != -2) ok = false;
        if (!ok) continue;
        agg[i] = na;
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
            if (strong(i, k)) agg[A.ci[k]] = na;
        ++na;
    }
    // pass 2: join the aggregate of the strongest aggregated neighbour
    std::vector<int64_t> pass2(n, -2);
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] != -2) continue;
        double best = 0.0;
        int64_t ba = -2;
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            if (!strong(i, k)) continue;
            const int64_t a = agg[A.ci[k]];
            if (a >= 0 && std::fabs(A.v[k]) > best) { best = std::fabs(A.v[k]); ba = a; }
        }
        pass2[i] = ba;
    }
    for (int64_t i = 0; i < n; ++i)
        if (agg[i] == -2 && pass2[i] >= 0) agg[i] = pass2[i];
    // pass 3: the rest aggregate with their free strong neighbours
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] != -2) continue;
        agg[i] = na;
        for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
            if (strong(i, k) && agg[A.ci[k]] == -2) agg[A.ci[k]] = na;
        ++na;
    }
    return na;
}

// Largest eigenvalue of D^-1 A by power iteration (upper estimate x 1.05).
double spectral_radius(const Csr &A, const std::vector<double> &dinv) {
    const int64_t n = A.n;
    std::vector<double> x(n), y(n);
    for (int64_t i = 0; i < n; ++i) x[i] = 1.0 + 0.37 * std::sin(1.7 * (double)i);
    double lam = 1.0;
    for (int it = 0; it < 20; ++it) {
        double nx = 0.0;
        for (int64_t i = 0; i < n; ++i) {
            double s = 0.0;
            for (int64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) s += A.v[k] * x[A.ci[k]];
            y[i] = dinv[i] * s;
            nx += y[i] * y[i];
        }
        nx = std::sqrt(nx);
        double xx = 0.0;
        for (int64_t i = 0; i < n; ++i) xx += x[i] * x[i];
        lam = nx / std::sqrt(xx);
        for (int64_t i = 0; i < n; ++i) x[i] = y[i] / nx;
    }
    return 1.05 * lam;
}

}  // namespace

int amg_setup(const Csr &A0, AmgHierarchy &h, bool constant_nullspace, const AmgParams &prm) {
    h.levels.clear();
    Csr A = A0;
    double theta = prm.theta;
    for (int lev = 0; lev < prm.max_levels; ++lev, theta *= prm.theta_factor) {
        AmgLevel L;
        L.A = A;
        const std::vector<double> d = diagonal(A);
        L.dinv.resize(A.n);
        for (int64_t i = 0; i < A.n; ++i) L.dinv[i] = d[i] != 0.0 ? 1.0 / d[i] : 1.0;
        const double rho = spectral_radius(A, L.dinv);
        L.omega = 4.0 / (3.0 * rho);   // smoother and prolongator smoothing weight
        if (A.n <= prm.coarse_max || lev == prm.max_levels - 1) {
            h.levels.push_back(L);
            break;
        }
        std::vector<int64_t> agg;
        const int64_t na = aggregate(A, d, theta, agg);
        if (na <= 0 || 2 * na > A.n) {   // coarsening stalls: this level is the coarsest
            h.levels.push_back(L);
            break;
        }
        // P0 then P = (I - omega D^-1 A) P0
        Csr P0;
        P0.n = A.n;
        P0.m = na;
        P0.rp.assign(A.n + 1, 0);
        for (int64_t i = 0; i < A.n; ++i) {
            if (agg[i] >= 0) { P0.ci.push_back((int32_t)agg[i]); P0.v.push_back(1.0); }
            P0.rp[i + 1] = (int64_t)P0.ci.size();
        }
        Csr AP0 = spgemm(A, P0);
        Csr P;
        P.n = A.n;
        P.m = na;
        P.rp.assign(A.n + 1, 0);
        std::vector<double> acc(na, 0.0);
        std::vector<int64_t> mark(na, -1);
        std::vector<int32_t> cols;
        for (int64_t i = 0; i < A.n; ++i) {
            cols.clear();
            for (int64_t k = P0.rp[i]; k < P0.rp[i + 1]; ++k) {
                const int32_t c = P0.ci[k];
                if (mark[c] != i) { mark[c] = i; acc[c] = 0.0; cols.push_back(c); }
                acc[c] += P0.v[k];
            }
            for (int64_t k = AP0.rp[i]; k < AP0.rp[i + 1]; ++k) {
                const int32_t c = AP0.ci[k];
                if (mark[c] != i) { mark[c] = i; acc[c] = 0.0; cols.push_back(c); }
                acc[c] -= L.omega * L.dinv[i] * AP0.v[k];
            }
            std::sort(cols.begin(), cols.end());
            for (int32_t c : cols)
                if (acc[c] != 0.0) { P.ci.push_back(c); P.v.push_back(acc[c]); }
            P.rp[i + 1] = (int64_t)P.ci.size();
        }
        L.R = transpose(P);
        Csr AP = spgemm(A, P);
        // S = (I - omega D^-1 A) P: one Jacobi sweep before and after the
        // coarse correction makes the V-cycle W + S B_c S^T
        L.S = P;
        {
            Csr SP;
            SP.n = A.n;
            SP.m = na;
            SP.rp.assign(A.n + 1, 0);
            for (int64_t i = 0; i < A.n; ++i) {
                cols.clear();
                for (int64_t k = P.rp[i]; k < P.rp[i + 1]; ++k) {
                    const int32_t c = P.ci[k];
                    if (mark[c] != A.n + i) { mark[c] = A.n + i; acc[c] = 0.0; cols.push_back(c); }
                    acc[c] += P.v[k];
                }
                for (int64_t k = AP.rp[i]; k < AP.rp[i + 1]; ++k) {
                    const int32_t c = AP.ci[k];
                    if (mark[c] != A.n + i) { mark[c] = A.n + i; acc[c] = 0.0; cols.push_back(c); }
                    acc[c] -= L.omega * L.dinv[i] * AP.v[k];
                }
                std::sort(cols.begin(), cols.end());
                for (int32_t c : cols)
                    if (acc[c] != 0.0) { SP.ci.push_back(c); SP.v.push_back(acc[c]); }
                SP.rp[i + 1] = (int64_t)SP.ci.size();
            }
            L.S = std::move(SP);
        }
        L.ST = transpose(L.S);
        L.P = P;
        A = spgemm(L.R, AP);
        h.levels.push_back(std::move(L));
    }
    // dense inverse of the coarsest operator (Gauss-Jordan, partial pivoting);
    // rows without entries get an identity row
    const Csr &C = h.levels.back().A;
    const int64_t nc = C.n;
    if (nc > prm.dense_max) return 9;
    std::vector<double> a(nc * nc, 0.0), inv(nc * nc, 0.0);
    for (int64_t i = 0; i < nc; ++i) {
        for (int64_t k = C.rp[i]; k < C.rp[i + 1]; ++k) a[i * nc + C.ci[k]] += C.v[k];
        inv[i * nc + i] = 1.0;
        if (a[i * nc + i] == 0.0) a[i * nc + i] = 1.0;
    }
    if (constant_nullspace && nc > 0) {
        // A_c 1 = 0 (smoothing keeps P 1 = 1 when A 1 = 0): invert A_c + (d/nc) 1 1^T,
        // d the mean diagonal, which is SPD and acts as A_c^+ on mean-free vectors
        double d = 0.0;
        for (int64_t i = 0; i < nc; ++i) d += a[i * nc + i];
        d /= (double)(nc * nc);
        for (int64_t k = 0; k < nc * nc; ++k) a[k] += d;
    }
    for (int64_t c = 0; c < nc; ++c) {
        int64_t piv = c;
        for (int64_t r = c + 1; r < nc; ++r)
            if (std::fabs(a[r * nc + c]) > std::fabs(a[piv * nc + c])) piv = r;
        if (a[piv * nc + c] == 0.0) return 8;
        if (piv != c)
            for (int64_t k = 0; k < nc; ++k) { std::swap(a[c * nc + k], a[piv * nc + k]); std::swap(inv[c * nc + k], inv[piv * nc + k]); }
        const double dd = a[c * nc + c];
        for (int64_t k = 0; k < nc; ++k) { a[c * nc + k] /= dd; inv[c * nc + k] /= dd; }
        for (int64_t r = 0; r < nc; ++r) {
            if (r == c) continue;
            const double f = a[r * nc + c];
            if (f == 0.0) continue;
            for (int64_t k = 0; k < nc; ++k) { a[r * nc + k] -= f * a[c * nc + k]; inv[r * nc + k] -= f * inv[c * nc + k]; }
        }
    }
    h.coarse_inv = inv;
    return 0;
}

void amg_cycle_operators(const AmgHierarchy &h, AmgCycle &c) {
    c = AmgCycle{};
    const int L = (int)h.levels.size() - 1;
    if (L < 1) return;
    const int64_t nL = h.levels[L].A.n;
    // G = C^-1 S_{L-1}^T: column j of G is C^-1 (row j of S_{L-1})
    const Csr &S = h.levels[L - 1].S;
    std::vector<double> g((size_t)nL * S.n, 0.0);
    for (int64_t j = 0; j < S.n; ++j)
        for (int64_t k = S.rp[j]; k < S.rp[j + 1]; ++k) {
            const int32_t col = S.ci[k];
            const double v = S.v[k];
            for (int64_t r = 0; r < nL; ++r) g[(size_t)r * S.n + j] += h.coarse_inv[(size_t)r * nL + col] * v;
        }
    c.G.n = nL;
    c.G.m = S.n;
    c.G.rp.assign(nL + 1, 0);
    for (int64_t r = 0; r < nL; ++r) {
        for (int64_t j = 0; j < S.n; ++j)
            if (g[(size_t)r * S.n + j] != 0.0) { c.G.ci.push_back((int32_t)j); c.G.v.push_back(g[(size_t)r * S.n + j]); }
        c.G.rp[r + 1] = (int64_t)c.G.ci.size();
    }
    c.stack_off.assign(L + 1, 0);
    if (L < 2) {
        c.stack_len = nL;
        return;
    }
    for (int l = 2; l <= L; ++l) c.stack_off[l] = l == 2 ? 0 : c.stack_off[l - 1] + h.levels[l - 1].A.n;
    c.stack_len = c.stack_off[L] + nL;
    // blocks Q_l = S_1 ... S_{l-1}, l = 2..L
    std::vector<Csr> Q;
    Q.push_back(h.levels[1].S);
    for (int l = 3; l <= L; ++l) Q.push_back(spgemm(Q.back(), h.levels[l - 1].S));
    const int64_t n1 = h.levels[1].A.n;
    c.U1.n = n1;
    c.U1.m = c.stack_len;
    c.U1.rp.assign(n1 + 1, 0);
    for (int64_t i = 0; i < n1; ++i) {
        for (int l = 2; l <= L; ++l) {
            const Csr &q = Q[l - 2];
            for (int64_t k = q.rp[i]; k < q.rp[i + 1]; ++k) {
                c.U1.ci.push_back((int32_t)(q.ci[k] + c.stack_off[l]));
                c.U1.v.push_back(q.v[k]);
            }
        }
        c.U1.rp[i + 1] = (int64_t)c.U1.ci.size();
    }
}

}  // namespace pg
