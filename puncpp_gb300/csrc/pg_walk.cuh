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

// Relative bound on |FP32 affine value - exact value| in units of the sum of
// the terms' magnitudes: one rounding per coefficient and per fmaf, with a
// factor two of slack.
constexpr float kPlaneEps = 8.0f * 5.9604645e-08f;   // 8 * 2^-24

// Barycentric coordinates of the FP32 point from a cell record's rows 0-2
// (the fourth is 1 - l0 - l1 - l2) and bounds on their FP32 errors.
__device__ __forceinline__ void lambdas_f32(const float4 r0, const float4 r1, const float4 r2, float x, float y,
                                            float z, float l[4], float e[4]) {
    const float4 r[3] = {r0, r1, r2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        l[k] = fmaf(r[k].w, z, fmaf(r[k].z, y, fmaf(r[k].y, x, r[k].x)));
        e[k] = kPlaneEps * (fabsf(r[k].x) + fabsf(r[k].y * x) + fabsf(r[k].z * y) + fabsf(r[k].w * z));
    }
    l[3] = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, l[0]), l[1]), l[2]);
    e[3] = e[0] + e[1] + e[2] + kPlaneEps * (1.0f + fabsf(l[0]) + fabsf(l[1]) + fabsf(l[2]));
}

// Is the FP32 point outside facet f (opposite local vertex f, where lambda_f
// = 0)?  Decided from the sign of lambda_f when it exceeds its error bound
// (lambda_f < 0 exactly when the facet's plane value is positive); otherwise
// re-tested in FP64 with the FP64 plane, the exact FP64 predicate at this
// point.
__device__ __forceinline__ bool facet_positive(const DevMesh &m, int c, int f, float l, float e, float x, float y,
                                               float z, int &retests) {
    if (l < -e) return true;
    if (l > e) return false;
    ++retests;
    const double2 *P = reinterpret_cast<const double2 *>(m.planes) + 8 * (size_t)c + 2 * f;
    const double2 a = __ldg(P), b = __ldg(P + 1);
    return plane64(a.x, a.y, b.x, b.y, (double)x, (double)y, (double)z) > 0;
}

// The walk of the mixed form: same facet order and semantics as walk_fp64,
// every decision equal to the FP64 predicate at the FP32 position.  Reads
// one 64-byte cell record per cell visited.
__device__ __forceinline__ int walk_mixed(const DevMesh &m, float x, float y, float z, int c, int max_steps,
                                          int &retests) {
    for (int it = 0; it < max_steps; ++it) {
        const float4 *R = m.cell_f + 4 * (size_t)c;
        const float4 r0 = __ldg(R), r1 = __ldg(R + 1), r2 = __ldg(R + 2), rn = __ldg(R + 3);
        float l[4], e[4];
        lambdas_f32(r0, r1, r2, x, y, z, l, e);
        int next;
        if (facet_positive(m, c, 0, l[0], e[0], x, y, z, retests)) next = __float_as_int(rn.x);
        else if (facet_positive(m, c, 1, l[1], e[1], x, y, z, retests)) next = __float_as_int(rn.y);
        else if (facet_positive(m, c, 2, l[2], e[2], x, y, z, retests)) next = __float_as_int(rn.z);
        else if (facet_positive(m, c, 3, l[3], e[3], x, y, z, retests)) next = __float_as_int(rn.w);
        else return c;
        if (next < 0) return next;
        c = next;
    }
    return kWalkFail;
}

// __float2ll_rn(v) for finite |v| < 2^62 on the 32-bit conversion path:
// below 2^23 in magnitude v rounds to nearest (even) in 32 bits; larger FP32
// values are integers, rebuilt from the significand and the exponent.
__device__ __forceinline__ long long float_to_ll_rn(float v) {
    if (fabsf(v) < 8388608.0f) return (long long)__float2int_rn(v);
    const unsigned u = __float_as_uint(v);
    const int sh = (int)((u >> 23) & 0xffu) - 150;
    const long long mag = (long long)((u & 0x7fffffu) | 0x800000u) << sh;
    return (u >> 31) ? -mag : mag;
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
// 2^-kFixedBits q_max (q_scaled = q * 2^kFixedBits / q_max in FP32), added with int64
// atomics, so the sum is the same in any order.
__device__ __forceinline__ void deposit_fixed(const DevMesh &m, int c, float x, float y, float z, float q_scaled,
                                              unsigned long long *rho_fixed) {
    const float4 *A = m.cell_f + 4 * (size_t)c;
    const float4 a0 = __ldg(A), a1 = __ldg(A + 1), a2 = __ldg(A + 2);
    const float l0 = fmaf(a0.w, z, fmaf(a0.z, y, fmaf(a0.y, x, a0.x)));
    const float l1 = fmaf(a1.w, z, fmaf(a1.z, y, fmaf(a1.y, x, a1.x)));
    const float l2 = fmaf(a2.w, z, fmaf(a2.z, y, fmaf(a2.y, x, a2.x)));
    const float l3 = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, l0), l1), l2);
    const int4 d = __ldg(m.dofs + c);
    atomicAdd(rho_fixed + d.x, (unsigned long long)float_to_ll_rn(__fmul_rn(l0, q_scaled)));
    atomicAdd(rho_fixed + d.y, (unsigned long long)float_to_ll_rn(__fmul_rn(l1, q_scaled)));
    atomicAdd(rho_fixed + d.z, (unsigned long long)float_to_ll_rn(__fmul_rn(l2, q_scaled)));
    atomicAdd(rho_fixed + d.w, (unsigned long long)float_to_ll_rn(__fmul_rn(l3, q_scaled)));
}

}  // namespace pg
