// Algebraic multigrid hierarchy (host side) of the Poisson preconditioner.
#pragma once

#include <cstdint>
#include <vector>

namespace pg {

struct Csr {
    int64_t n = 0, m = 0;            // rows, columns
    std::vector<int64_t> rp;         // [n+1]
    std::vector<int32_t> ci;
    std::vector<double> v;
};

struct AmgLevel {
    Csr A;                           // level operator
    Csr P, R;                        // prolongator to this level from the next, R = P^T (empty on the coarsest)
    Csr S, ST;                       // (I - omega D^-1 A) P and its transpose: the V-cycle's transfer operators
    std::vector<double> dinv;        // D^-1
    double omega = 0.0;              // Jacobi weight 4 / (3 rho(D^-1 A))
};

struct AmgParams {
    double theta = 0.0;              // strength threshold on level 0 (0: every coupling is strong)
    double theta_factor = 1.0;       // theta on level l = theta * theta_factor^l
    int64_t coarse_max = 400;        // coarsen until at most this many rows
    int64_t dense_max = 4096;        // largest coarsest level inverted densely
    int max_levels = 12;
};

struct AmgHierarchy {
    std::vector<AmgLevel> levels;
    std::vector<double> coarse_inv;  // dense inverse of the coarsest operator
};

// Operators of the device cycle, for L = levels - 1 >= 1 levels above the
// coarsest: G = C^-1 S_{L-1}^T (n_L x n_{L-1}, the last restriction and the
// coarse solve in one product) and, when L >= 2, the collapsed up-sweep of
// levels 1..L-1,
//     y_1 = t_1 + U1 [t_2; ...; t_{L-1}; y_L],
//     U1 = [S_1 | S_1 S_2 | ... | S_1 ... S_{L-1}],
// acting on the stacked vector whose level-l block starts at stack_off[l]
// (l = 2..L; for L = 1, y_1 = G b_0 is the whole stack).
struct AmgCycle {
    Csr G, U1;
    std::vector<int64_t> stack_off;  // [L + 1], entries 0, 1 unused
    int64_t stack_len = 0;
};
void amg_cycle_operators(const AmgHierarchy &h, AmgCycle &c);

// Returns 0; 8 when the coarsest operator is singular; 9 when coarsening
// stalls above AmgParams::dense_max rows.  With
// `constant_nullspace` (periodic meshes: A 1 = 0) the coarsest inverse is
// that of A_c + (mean diag / n_c) 1 1^T.
int amg_setup(const Csr &A0, AmgHierarchy &h, bool constant_nullspace, const AmgParams &prm = AmgParams());

}  // namespace pg
