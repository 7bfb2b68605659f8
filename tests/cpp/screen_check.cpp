// Checks the FP32 screen of the flux rejection test (pg_screen.h) against the
// exact FP64 test: on random candidates and on candidates whose test uniform
// is placed at relative distances 1e-9 .. 1e-2 from the acceptance boundary,
// the screen must never answer accept or reject where the FP64 test says the
// opposite.  Prints: candidates, contradictions, undecided, random candidates,
// undecided random candidates.
#include <cmath>
#include <cstdint>
#include <cstdio>

#include "pg_screen.h"

using namespace pg;

// words (x, y) with u01_from(x, y) = floor(u 2^53) / 2^53
static void words_of(double u, uint32_t &x, uint32_t &y) {
    const uint64_t N = (uint64_t)std::floor(u * 9007199254740992.0);
    x = (uint32_t)((N >> 26) << 5);
    y = (uint32_t)((N & ((1ull << 26) - 1)) << 6);
}

int main() {
    long long total = 0, bad = 0, undecided = 0, random_total = 0, random_undecided = 0;
    const double vths[3] = {1.0, 0.0233, 3.7};
    const double drifts[3][3] = {{0, 0, 0}, {0.4, -0.2, 0.1}, {-2.5, 1.0, 0.0}};
    const double normals[4][3] = {{1, 0, 0}, {0, -1, 0}, {0.57735026918962573, 0.57735026918962573, -0.57735026918962573},
                                  {0.28, -0.96, 0.0}};
    uint32_t ctr = 0;
    for (double vth : vths)
        for (const auto &vd : drifts)
            for (const auto &n : normals) {
                FluxBox B;
                for (int c = 0; c < 3; ++c) {
                    B.lo[c] = vd[c] - 5.0 * vth;
                    B.w[c] = 10.0 * vth;
                    B.vd[c] = vd[c];
                }
                B.vth2 = vth * vth;
                B.factor = 1.0 / std::pow(std::sqrt(2.0 * M_PI * B.vth2), 3);
                // pdf_max over a grid of the box (any positive bound works)
                double pmax = 0.0, t[3];
                for (int i = 0; i <= 40; ++i)
                    for (int j = 0; j <= 40; ++j)
                        for (int k = 0; k <= 40; ++k) {
                            flux_accept_fp64(B, n[0], n[1], n[2], 0.0, i / 40.0, j / 40.0, k / 40.0, 2.0, t);
                            double vn = t[0] * n[0] + t[1] * n[1] + t[2] * n[2];
                            double vs = 0;
                            for (int c = 0; c < 3; ++c) vs += (t[c] - vd[c]) * (t[c] - vd[c]);
                            const double p = (vn > 0) * vn * B.factor * std::exp(-0.5 * vs / B.vth2);
                            if (p > pmax) pmax = p;
                        }
                const FluxBox32 F = flux_box32(B);
                for (int m = 0; m < 20000; ++m) {
                    const Philox4 ra = philox4x32_10(ctr, 7u, 11u, 13u, 0x1234u, 0x5678u);
                    const Philox4 rb = philox4x32_10(ctr, 8u, 11u, 13u, 0x1234u, 0x5678u);
                    ++ctr;
                    const double a = u01_from(ra.v[0], ra.v[1]), b = u01_from(ra.v[2], ra.v[3]);
                    const double c = u01_from(rb.v[0], rb.v[1]);
                    // the candidate's exact pdf, to place u near the boundary
                    double tt[3];
                    flux_accept_fp64(B, n[0], n[1], n[2], 1.0, a, b, c, 2.0, tt);
                    double vn = 0.0;
                    vn += tt[0] * n[0]; vn += tt[1] * n[1]; vn += tt[2] * n[2];
                    double vs = 0.0;
                    for (int q = 0; q < 3; ++q) vs += (tt[q] - vd[q]) * (tt[q] - vd[q]);
                    const double pdf = (double)(vn > 0.0) * vn * (B.factor * exp_portable(-0.5 * vs / B.vth2));
                    for (int v = 0; v < 9; ++v) {
                        uint32_t xu, yu;
                        if (v == 0) {
                            xu = rb.v[2];
                            yu = rb.v[3];
                        } else {
                            const double rel = std::pow(10.0, -9.0 + (v - 1)) * ((v & 1) ? 1.0 : -1.0);
                            double u = pdf / pmax * (1.0 + rel);
                            if (!(u >= 0.0 && u < 1.0)) continue;
                            words_of(u, xu, yu);
                        }
                        const double u = u01_from(xu, yu);
                        const bool exact = flux_accept_fp64(B, n[0], n[1], n[2], pmax, a, b, c, u, tt);
                        const int s = flux_screen_fp32(F, (float)n[0], (float)n[1], (float)n[2], (float)pmax, ra.v[0],
                                                       ra.v[2], rb.v[0], xu);
                        ++total;
                        if (v == 0) { ++random_total; random_undecided += s < 0; }
                        if (s < 0) ++undecided;
                        else if ((s == 1) != exact) ++bad;
                    }
                }
            }
    std::printf("%lld %lld %lld %lld %lld\n", total, bad, undecided, random_total, random_undecided);
    return bad == 0 ? 0 : 1;
}
