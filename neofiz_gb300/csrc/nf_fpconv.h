// nf_fpconv.h -- float <-> double conversions in 32-bit integer arithmetic, bit for bit the
// IEEE round-to-nearest-even conversions.
//
// On GB300 a conversion between float and double issues on the FP64 pipe, like an FP64 add: the
// mixed form's gather, which widened each float contribution before adding it in double, ran
// half its FP64-pipe instructions as conversions, and took 49 us a step on a 1M-quad scene where
// the FP64 gather, reading twice the bytes, took 33 us (31 us with the widening below). The
// mixed form converted about twenty values per node and step (a node's positions as float pairs
// and v dt, and its force contributions). These forms take a few 32-bit integer operations
// each.
//
// Each function returns the bit pattern the conversion gives. The split and the narrowing cover
// the ranges the geometry of a scene lives in and return false outside them (the caller then
// converts); the widening covers every float (a NaN gives a quiet NaN). Host and device compile
// the same code, so the host checks it against the C conversions.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define NF_CONV_FN __host__ __device__ __forceinline__
#else
#define NF_CONV_FN static inline
#endif

// Bit length of a nonzero 32-bit value.
NF_CONV_FN int nf_bitlen32(uint32_t a) {
#ifdef __CUDA_ARCH__
    return 32 - __clz((int)a);
#else
    return 32 - __builtin_clz(a);
#endif
}

// Round a (bit length nb in 25..31) to its top 24 bits, nearest, ties to even; the result is in
// [2^23, 2^24] (2^24 when the rounding carries, which the exponent arithmetic below absorbs).
NF_CONV_FN uint32_t nf_round24(uint32_t a, int nb) {
    const int s = nb - 24;
    const uint32_t keep = a >> s, rem = a & ((1u << s) - 1u), half = 1u << (s - 1);
    return keep + ((rem > half || (rem == half && (keep & 1u))) ? 1u : 0u);
}

// The double with high word hw and low word lw, x = (-1)^s M 2^(E-52) with M the 53-bit
// significand: RN(x) to binary32 keeps M's top 24 bits, rounded on the 29 below them. A carry
// into 2^24 adds one to the exponent field through the sum ((e - 1) << 23) + keep, where keep
// still holds the implicit bit.
NF_CONV_FN uint32_t nf_round_top24(uint32_t hw, uint32_t lw, uint32_t &rem29, uint32_t &up) {
    const uint32_t keep = (((hw & 0xfffffu) | 0x100000u) << 3) | (lw >> 29);
    rem29 = lw & 0x1fffffffu;
    up = (rem29 > 0x10000000u || (rem29 == 0x10000000u && (keep & 1u))) ? 1u : 0u;
    return keep + up;
}

// RN(x) for 2^-126 <= |x| < 2^127 (a normal float that cannot overflow) or x = +-0.
NF_CONV_FN bool nf_narrow_bits(uint32_t hw, uint32_t lw, uint32_t &out) {
    const uint32_t sign = hw & 0x80000000u, ed = (hw >> 20) & 0x7ffu;
    if ((hw & 0x7fffffffu) == 0u && lw == 0u) {
        out = sign;
        return true;
    }
    if (ed < 897u || ed > 1149u) return false;
    uint32_t rem, up;
    const uint32_t keep = nf_round_top24(hw, lw, rem, up);
    out = sign | (((ed - 897u) << 23) + keep);      // float exponent field ed - 896
    return true;
}

// hi = RN(x) and lo = RN(x - hi), as the expressions (float)x and (float)(x - (double)(float)x)
// give them, for 2^-74 <= |x| < 2^127 or x = +-0. x - hi is exact in double: it is r 2^(E-52)
// with r = M - keep 2^29, |r| <= 2^28; lo rounds r to 24 bits, and its exponent field is
// ed + bitlen(r) - 949, at least 1 in this range. x = +-0 gives hi = x and lo = +0, as x - x
// is +0 for either zero.
NF_CONV_FN bool nf_split_bits(uint32_t hw, uint32_t lw, uint32_t &hi, uint32_t &lo) {
    const uint32_t sign = hw & 0x80000000u, ed = (hw >> 20) & 0x7ffu;
    if ((hw & 0x7fffffffu) == 0u && lw == 0u) {
        hi = sign;
        lo = 0u;
        return true;
    }
    if (ed < 949u || ed > 1149u) return false;
    uint32_t rem, up;
    const uint32_t keep = nf_round_top24(hw, lw, rem, up);
    hi = sign | (((ed - 897u) << 23) + keep);
    const int32_t r = (int32_t)rem - (up ? 0x20000000 : 0);
    if (r == 0) {
        lo = 0u;
        return true;
    }
    const uint32_t a = r < 0 ? (uint32_t)(-r) : (uint32_t)r;
    const int nb = nf_bitlen32(a);
    const uint32_t m = nb <= 24 ? a << (24 - nb) : nf_round24(a, nb);
    lo = (sign ^ (r < 0 ? 0x80000000u : 0u)) | (((ed + (uint32_t)nb - 950u) << 23) + m);
    return true;
}

// (double)f for the float with bits u, as the double's high and low words: exact for every
// float; a NaN keeps its payload and is made quiet.
NF_CONV_FN void nf_widen_words(uint32_t u, uint32_t &hw, uint32_t &lw) {
    const uint32_t sign = u & 0x80000000u, a = u & 0x7fffffffu;
    if (a >= 0x00800000u && a < 0x7f800000u) {      // normal: rebias the exponent by 896
        hw = sign | ((a >> 3) + (896u << 20));
        lw = a << 29;
    } else if (a == 0u) {
        hw = sign;
        lw = 0u;
    } else if (a >= 0x7f800000u) {                  // infinity, NaN
        hw = sign | 0x7ff00000u | (a > 0x7f800000u ? 0x00080000u : 0u) | ((a & 0x7fffffu) >> 3);
        lw = a << 29;
    } else {                                        // subnormal a 2^-149: normalise
        const int nb = nf_bitlen32(a);              // 1..23; exponent field nb + 873
        const uint64_t frac = (uint64_t)(a ^ (1u << (nb - 1))) << (53 - nb);
        hw = sign | (((uint32_t)nb + 873u) << 20) | (uint32_t)(frac >> 32);
        lw = (uint32_t)frac;
    }
}

#ifdef __CUDACC__
// The device forms: the integer conversion where it applies, the instruction elsewhere.
__device__ __forceinline__ double nf_widen(float f) {
    uint32_t hw, lw;
    nf_widen_words(__float_as_uint(f), hw, lw);
    return __hiloint2double((int)hw, (int)lw);
}
__device__ __forceinline__ float nf_narrow(double x) {
    uint32_t b;
    if (nf_narrow_bits((uint32_t)__double2hiint(x), (uint32_t)__double2loint(x), b))
        return __uint_as_float(b);
    return (float)x;
}
__device__ __forceinline__ float2 nf_split(double x) {
    uint32_t h, l;
    if (nf_split_bits((uint32_t)__double2hiint(x), (uint32_t)__double2loint(x), h, l))
        return make_float2(__uint_as_float(h), __uint_as_float(l));
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}
#endif
