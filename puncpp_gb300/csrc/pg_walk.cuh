// Device routines shared by the particle, injection and mixed-precision
// kernels: the facet walk, barycentric coordinates and the fixed-point
// deposit.  Every FP64 product and sum is an explicit round-to-nearest
// intrinsic and every FP32 one an explicit fmaf or __f*_rn, so the results do
// not depend on the translation unit's --fmad setting.
#pragma once

#include "pg_device.cuh"

namespace pg {

__device__ __forceinline__ void raise_device_error(DevState *st, int code, int64_t idx) {
    if (atomicCAS(&st->err_code, 0, code) == 0) st->err_index = idx;
}

// c0 + c1 x + c2 y + c3 z summed left to right with each step rounded, as
// relocate_fast evaluates it (punc/include/punc/population.h:549-552).
__device__ __forceinline__ double plane64(double c0, double c1, double c2, double c3, double x, double y, double z) {
    double d = __dadd_rn(c0, __dmul_rn(c1, x));
    d = __dadd_rn(d, __dmul_rn(c2, y));
    return __dadd_rn(d, __dmul_rn(c3, z));
}

// relocate_fast (punc/include/punc/population.h:539-569) as a bounded loop:
// the first facet i (0..3) with a positive plane value moves the walk to
// neighbour i or ends it with -tag; no positive facet ends it in the cell.
__device__ __forceinline__ int walk_fp64(const DevMesh &m, double x, double y, double z, int c, int max_steps) {
    for (int it = 0; it < max_steps; ++it) {
        const double2 *P = reinterpret_cast<const double2 *>(m.planes) + 8 * (size_t)c;
        const double2 q0 = __ldg(P + 0), q1 = __ldg(P + 1), q2 = __ldg(P + 2), q3 = __ldg(P + 3);
        const double2 q4 = __ldg(P + 4), q5 = __ldg(P + 5), q6 = __ldg(P + 6), q7 = __ldg(P + 7);
        const int4 nb = __ldg(m.nbr + c);
        const double d0 = plane64(q0.x, q0.y, q1.x, q1.y, x, y, z);
        const double d1 = plane64(q2.x, q2.y, q3.x, q3.y, x, y, z);
        const double d2 = plane64(q4.x, q4.y, q5.x, q5.y, x, y, z);
        const double d3 = plane64(q6.x, q6.y, q7.x, q7.y, x, y, z);
        int next;
        if (d0 > 0) next = nb.x;
        else if (d1 > 0) next = nb.y;
        else if (d2 > 0) next = nb.z;
        else if (d3 > 0) next = nb.w;
        else return c;
        if (next < 0) return next;
        c = next;
    }
    return kWalkFail;
}

// Relative bound on |FP32 plane value - exact value| in units of the sum of
// the terms' magnitudes: one rounding per coefficient and per fmaf, with a
// factor two of slack.
constexpr float kPlaneEps = 8.0f * 5.9604645e-08f;   // 8 * 2^-24

// Sign of facet f's plane value at the FP32 point, decided in FP32 unless the
// value is within the error bound of zero, then re-tested in FP64 with the
// FP64 plane (the exact FP64 predicate at this point).
__device__ __forceinline__ bool facet_positive(const DevMesh &m, int c, int f, float4 pl, float x, float y, float z,
                                               int &retests) {
    const float d = fmaf(pl.w, z, fmaf(pl.z, y, fmaf(pl.y, x, pl.x)));
    const float s = fabsf(pl.x) + fabsf(pl.y * x) + fabsf(pl.z * y) + fabsf(pl.w * z);
    const float e = kPlaneEps * s;
    if (d > e) return true;
    if (d < -e) return false;
    ++retests;
    const double2 *P = reinterpret_cast<const double2 *>(m.planes) + 8 * (size_t)c + 2 * f;
    const double2 a = __ldg(P), b = __ldg(P + 1);
    return plane64(a.x, a.y, b.x, b.y, (double)x, (double)y, (double)z) > 0;
}

// The walk of the mixed form: same facet order and semantics as walk_fp64,
// every decision equal to the FP64 predicate at the FP32 position.
__device__ __forceinline__ int walk_mixed(const DevMesh &m, float x, float y, float z, int c, int max_steps,
                                          int &retests) {
    for (int it = 0; it < max_steps; ++it) {
        const float4 *P = reinterpret_cast<const float4 *>(m.planes_f) + 4 * (size_t)c;
        const int4 nb = __ldg(m.nbr + c);
        int next;
        if (facet_positive(m, c, 0, __ldg(P + 0), x, y, z, retests)) next = nb.x;
        else if (facet_positive(m, c, 1, __ldg(P + 1), x, y, z, retests)) next = nb.y;
        else if (facet_positive(m, c, 2, __ldg(P + 2), x, y, z, retests)) next = nb.z;
        else if (facet_positive(m, c, 3, __ldg(P + 3), x, y, z, retests)) next = nb.w;
        else return c;
        if (next < 0) return next;
        c = next;
    }
    return kWalkFail;
}

// Cell<3>::barycentric (punc/include/punc/population.h:885-893), FP64.
__device__ __forceinline__ void barycentric_fp64(const DevMesh &m, int c, double x, double y, double z,
                                                 double &l0, double &l1, double &l2, double &l3) {
    const double2 *A = reinterpret_cast<const double2 *>(m.bary) + 6 * (size_t)c;
    const double2 a0 = __ldg(A + 0), a1 = __ldg(A + 1), a2 = __ldg(A + 2);
    const double2 a3 = __ldg(A + 3), a4 = __ldg(A + 4), a5 = __ldg(A + 5);
    l0 = plane64(a0.x, a0.y, a1.x, a1.y, x, y, z);
    l1 = plane64(a2.x, a2.y, a3.x, a3.y, x, y, z);
    l2 = plane64(a4.x, a4.y, a5.x, a5.y, x, y, z);
    l3 = __dadd_rn(__dadd_rn(__dadd_rn(1.0, -l0), -l1), -l2);
}

// Fixed-point CG1 deposit of the mixed form: q*lambda_i in units of
// 2^-40 q_max (q_scaled = q * 2^40 / q_max in FP32), added with int64
// atomics, so the sum is the same in any order.
__device__ __forceinline__ void deposit_fixed(const DevMesh &m, int c, float x, float y, float z, float q_scaled,
                                              unsigned long long *rho_fixed) {
    const float4 *A = reinterpret_cast<const float4 *>(m.bary_f) + 3 * (size_t)c;
    const float4 a0 = __ldg(A), a1 = __ldg(A + 1), a2 = __ldg(A + 2);
    const float l0 = fmaf(a0.w, z, fmaf(a0.z, y, fmaf(a0.y, x, a0.x)));
    const float l1 = fmaf(a1.w, z, fmaf(a1.z, y, fmaf(a1.y, x, a1.x)));
    const float l2 = fmaf(a2.w, z, fmaf(a2.z, y, fmaf(a2.y, x, a2.x)));
    const float l3 = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, l0), l1), l2);
    const int4 d = __ldg(m.dofs + c);
    atomicAdd(rho_fixed + d.x, (unsigned long long)__float2ll_rn(__fmul_rn(l0, q_scaled)));
    atomicAdd(rho_fixed + d.y, (unsigned long long)__float2ll_rn(__fmul_rn(l1, q_scaled)));
    atomicAdd(rho_fixed + d.z, (unsigned long long)__float2ll_rn(__fmul_rn(l2, q_scaled)));
    atomicAdd(rho_fixed + d.w, (unsigned long long)__float2ll_rn(__fmul_rn(l3, q_scaled)));
}

}  // namespace pg
