// Rejection test of the flux sampler (punc/src/injector.cpp:51-76): candidate
// velocity t = lo + w (a, b, c) in the box vd +- range vth, accepted when
//     u pdf_max < max(t.n, 0) factor exp(-|t - vd|^2 / (2 vth^2)).
//
// flux_accept_fp64 is the exact test in the oracle's FP64 arithmetic (no
// contraction).  flux_screen_fp32 decides the same test in FP32 from the same
// random words, with a bound on the difference between its FP32 values and the
// FP64 ones; it answers accept or reject only when the FP32 margin exceeds the
// bound, and "undecided" otherwise, so that a caller who falls back to the
// FP64 test for undecided candidates takes exactly the FP64 decisions.
//
// Error bound (e = 2^-24, every FP32 operation rounds once, expf within 2 ulp):
//   t_c:    4e (|lo_c| + |w_c| + |t_c|)     (a in FP32 is a truncated to 24
//                                            bits; lo, w rounded to FP32)
//   t.n:    sum |n_c| dt_c + 8e sum |t_c n_c|   (n rounded to FP32, five roundings)
//   d = t - vd, |d|^2: sum (2 |d_c| dd_c + dd_c^2) + 4e |d|^2,
//           dd_c = dt_c + 2e (|vd_c| + |d_c|)
//   arg = -h |d|^2, h = 1 / (2 vth^2):  h d(|d|^2) + 4e |arg|
//   f = factor exp(arg):  relative 1.01 d(arg) + 8e
//   pdf = (t.n) f:  f (1 + rel_f) d(t.n) + |pdf| (rel_f + 2e)
//   u pdf_max:      4e pdf_max
// and the decision margin is twice their sum (twice d(t.n) for the sign of
// t.n).  Candidates with
// f < 1e-30 (near FP32 underflow) or d(arg) > 1e-2 are undecided.
#pragma once

#include <cmath>
#include <cstdint>

#include "pg_math.h"

namespace pg {

struct FluxBox {
    double lo[3], w[3], vd[3];
    double vth2, factor;
};

// Exact test; returns the candidate velocity in t.
PG_HD bool flux_accept_fp64(const FluxBox &B, double nx, double ny, double nz, double pmax, double a, double b,
                            double c, double u, double t[3]) {
    t[0] = B.lo[0] + B.w[0] * a;
    t[1] = B.lo[1] + B.w[1] * b;
    t[2] = B.lo[2] + B.w[2] * c;
    double vn = 0.0;
    vn += t[0] * nx; vn += t[1] * ny; vn += t[2] * nz;
    double vs = 0.0;
    vs += (t[0] - B.vd[0]) * (t[0] - B.vd[0]);
    vs += (t[1] - B.vd[1]) * (t[1] - B.vd[1]);
    vs += (t[2] - B.vd[2]) * (t[2] - B.vd[2]);
    const double f = B.factor * exp_portable(-0.5 * vs / B.vth2);
    const double pdf = (double)(vn > 0.0) * vn * f;
    return u * pmax < pdf;
}

// The FP32 copies of a box (set up once per particle).
struct FluxBox32 {
    float lo[3], w[3], vd[3];
    float bt[3];      // 4e (|lo| + |w|): the part of dt_c independent of t
    float vdabs[3];   // |vd|
    float h, factor;
};

PG_HD FluxBox32 flux_box32(const FluxBox &B) {
    const float e = 5.9604645e-08f;   // 2^-24
    FluxBox32 F;
    for (int k = 0; k < 3; ++k) {
        F.lo[k] = (float)B.lo[k];
        F.w[k] = (float)B.w[k];
        F.vd[k] = (float)B.vd[k];
        F.bt[k] = 4.0f * e * ((float)std::fabs(B.lo[k]) + (float)std::fabs(B.w[k]));
        F.vdabs[k] = (float)std::fabs(B.vd[k]);
    }
    F.h = (float)(0.5 / B.vth2);
    F.factor = (float)B.factor;
    return F;
}

// 24-bit truncation of u01_from(x, .): the top 24 of its 53 bits.
PG_HD float u01_24(uint32_t x) { return (float)(x >> 8) * 5.9604645e-08f; }

// 1 accept, 0 reject, -1 undecided; xa, xb, xc, xu are the first words of the
// four uniforms (u01_from(xa, .) = a, ...).
PG_HD int flux_screen_fp32(const FluxBox32 &F, float nx, float ny, float nz, float pmax, uint32_t xa, uint32_t xb,
                           uint32_t xc, uint32_t xu) {
    const float e = 5.9604645e-08f;
    const float n[3] = {nx, ny, nz};
    const float r[3] = {u01_24(xa), u01_24(xb), u01_24(xc)};
    float t[3], dt[3];
    for (int k = 0; k < 3; ++k) {
        t[k] = F.lo[k] + F.w[k] * r[k];
        dt[k] = F.bt[k] + 4.0f * e * std::fabs(t[k]);
    }
    const float vn = t[0] * n[0] + t[1] * n[1] + t[2] * n[2];
    const float dvn = std::fabs(n[0]) * dt[0] + std::fabs(n[1]) * dt[1] + std::fabs(n[2]) * dt[2] +
                      8.0f * e * (std::fabs(t[0] * n[0]) + std::fabs(t[1] * n[1]) + std::fabs(t[2] * n[2]));
    if (vn + 2.0f * dvn <= 0.0f) return 0;   // t.n <= 0: pdf = 0 and u pdf_max >= 0
    if (vn - 2.0f * dvn <= 0.0f) return -1;
    float vs = 0.0f, dvs = 0.0f;
    for (int k = 0; k < 3; ++k) {
        const float d = t[k] - F.vd[k];
        const float dd = dt[k] + 2.0f * e * (F.vdabs[k] + std::fabs(d));
        vs += d * d;
        dvs += 2.0f * std::fabs(d) * dd + dd * dd;
    }
    dvs += 4.0f * e * vs;
    const float arg = -F.h * vs;
    const float darg = F.h * dvs + 4.0f * e * std::fabs(arg);
    if (!(darg <= 1e-2f)) return -1;
    const float f = F.factor * expf(arg);
    if (!(f >= 1e-30f)) return -1;
    const float relf = 1.01f * darg + 8.0f * e;
    const float pdf = vn * f;
    const float dpdf = f * (1.0f + relf) * dvn + pdf * (relf + 2.0f * e);
    const float L = u01_24(xu) * pmax;
    const float margin = 2.0f * (dpdf + 4.0f * e * pmax);
    if (L < pdf - margin) return 1;
    if (L > pdf + margin) return 0;
    return -1;
}

}  // namespace pg
