// Host/device helpers whose results must be bitwise identical on the CPU and
// the GPU: the Philox4x32-10 counter-based generator and an exp() written
// from its Taylor series.  Compile every user of this header without
// floating-point contraction (host: -ffp-contract=off, device: --fmad=false).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PG_HD __host__ __device__ __forceinline__
#else
#define PG_HD inline
#endif

namespace pg {

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with a
// Weyl-sequence key schedule.
struct Philox4 {
    uint32_t v[4];
};

PG_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
    const uint64_t p = uint64_t(a) * uint64_t(b);
    hi = uint32_t(p >> 32);
    lo = uint32_t(p);
}

PG_HD Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
    for (int round = 0; round < 10; ++round) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c0, hi0, lo0);
        mulhilo32(0xCD9E8D57u, c2, hi1, lo1);
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    Philox4 r;
    r.v[0] = c0; r.v[1] = c1; r.v[2] = c2; r.v[3] = c3;
    return r;
}

// 53-bit uniform double in [0,1) from two 32-bit words (the res53 recipe of
// Matsumoto and Nishimura's MT19937 reference code).
PG_HD double u01_from(uint32_t a, uint32_t b) {
    return (double(a >> 5) * 67108864.0 + double(b >> 6)) * (1.0 / 9007199254740992.0);
}

// A sequential stream of uniforms: stream id (c1, c2, c3) plus a draw counter.
// Each Philox block yields two doubles.
struct Stream {
    uint32_t key0, key1, c1, c2, c3;
    uint32_t block;
    int have;        // 0 or 1 cached uniforms
    double cached;
    PG_HD void init(uint64_t seed, uint32_t s1, uint32_t s2, uint32_t s3) {
        key0 = uint32_t(seed); key1 = uint32_t(seed >> 32);
        c1 = s1; c2 = s2; c3 = s3; block = 0; have = 0; cached = 0.0;
    }
    PG_HD double next() {
        if (have) { have = 0; return cached; }
        const Philox4 r = philox4x32_10(block, c1, c2, c3, key0, key1);
        ++block;
        cached = u01_from(r.v[2], r.v[3]);
        have = 1;
        return u01_from(r.v[0], r.v[1]);
    }
};

// exp(x): x = k ln2 + r with |r| <= ln2/2 (ln2 split in a 24-bit head and a
// tail so k*head is exact), e^r from its Taylor series to r^13 by Horner's
// rule, then scaled by 2^k built from the exponent bits.
PG_HD double exp_portable(double x) {
    if (x != x) return x;
    if (x > 709.5) return HUGE_VAL;
    if (x < -745.0) return 0.0;
    const double inv_ln2 = 0x1.71547652b82fep+0;
    const double ln2_hi = 0x1.62e4300000000p-1;
    const double ln2_lo = -0x1.05c610ca86c39p-29;
    const double kf = floor(x * inv_ln2 + 0.5);
    const double r = (x - kf * ln2_hi) - kf * ln2_lo;
    double p = 0x1.6124613a86d09p-33;        // 1/13!
    p = p * r + 0x1.1eed8eff8d898p-29;       // 1/12!
    p = p * r + 0x1.ae64567f544e4p-26;       // 1/11!
    p = p * r + 0x1.27e4fb7789f5cp-22;       // 1/10!
    p = p * r + 0x1.71de3a556c734p-19;       // 1/9!
    p = p * r + 0x1.a01a01a01a01ap-16;       // 1/8!
    p = p * r + 0x1.a01a01a01a01ap-13;       // 1/7!
    p = p * r + 0x1.6c16c16c16c17p-10;       // 1/6!
    p = p * r + 0x1.1111111111111p-7;        // 1/5!
    p = p * r + 0x1.5555555555555p-5;        // 1/4!
    p = p * r + 0x1.5555555555555p-3;        // 1/3!
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    int k = int(kf);
    // 2^k as a double; split when the result would be subnormal.
    double scale_extra = 1.0;
    if (k < -1020) { k += 1000; scale_extra = 0x1p-1000; }
    const uint64_t bits = uint64_t(int64_t(k) + 1023) << 52;
#ifdef __CUDA_ARCH__
    const double two_k = __longlong_as_double((long long)bits);
#else
    double two_k;
    std::memcpy(&two_k, &bits, sizeof(double));
#endif
    return (p * two_k) * scale_extra;
}

}  // namespace pg
