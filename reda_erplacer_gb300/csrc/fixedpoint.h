// Conversions between FP32 and the 64-bit fixed-point density sums, in 32-bit
// integer arithmetic only.  Both round to nearest, ties to even, exactly like
// __float2ll_rn / __ll2float_rn on their ranges, but conversions to and from
// 64-bit types issue on the FP64 pipe, which runs at a small fraction of the
// FP32 rate on GB300; the density scatter converts every (cell, bin)
// contribution and the row pass every bin.
//
// The header compiles for the device and for the host, so that a host program
// can check the routines against the C library's conversions.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define ERP_FXP_FN __host__ __device__ __forceinline__
#else
#define ERP_FXP_FN static inline
#endif

namespace erp {

ERP_FXP_FN uint32_t fxp_float_bits(float v) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(v);
#else
    uint32_t b;
    memcpy(&b, &v, sizeof b);
    return b;
#endif
}

ERP_FXP_FN float fxp_bits_float(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float v;
    memcpy(&v, &b, sizeof v);
    return v;
#endif
}

ERP_FXP_FN int fxp_clz32(uint32_t x) {   // x != 0
#if defined(__CUDA_ARCH__)
    return __clz((int)x);
#else
    return __builtin_clz(x);
#endif
}

// rint(v) for v in [0, 2^63) (round half to even).  Outside that range
// (negative, >= 2^63, infinite or NaN: the caller's error) the result is 0.
// A float of exponent field e holds the integer mantissa m (24 bits with the
// hidden one) times 2^(e - 150).
ERP_FXP_FN uint64_t fxp_rint_u64(float v) {
    const uint32_t b = fxp_float_bits(v);
    if (b >> 31) return 0;
    const int e = (int)(b >> 23);
    if (e < 126 || e >= 190) return 0;   // v < 0.5 (zero and subnormals included), or v >= 2^63
    const uint32_t m = (b & 0x7fffffu) | 0x800000u;
    if (e >= 150) return (uint64_t)m << (e - 150);   // already an integer
    const int sh = 150 - e;   // 1 .. 24
    uint32_t q = m >> sh;
    const uint32_t rem = m & ((1u << sh) - 1u), half = 1u << (sh - 1);
    q += (rem > half || (rem == half && (q & 1u))) ? 1u : 0u;
    return q;
}

// (float)q, round half to even, for any q < 2^64.
ERP_FXP_FN float fxp_u64_to_float(uint64_t q) {
    const uint32_t hi = (uint32_t)(q >> 32), lo = (uint32_t)q;
    if (hi == 0 && lo == 0) return 0.0f;
    // normalise the top set bit to bit 31 of `top`; the bits below the 24
    // kept ones decide the rounding
    int lz;
    uint32_t top, rest;   // rest: the bits below `top`, nonzero-ness only
    if (hi) {
        lz = fxp_clz32(hi);
        top = lz ? (hi << lz) | (lo >> (32 - lz)) : hi;
        rest = lz ? (lo << lz) : lo;
    } else {
        lz = 32 + fxp_clz32(lo);
        top = lo << (lz - 32);
        rest = 0;
    }
    const int e = 63 - lz;                  // q in [2^e, 2^(e+1))
    uint32_t mant = top >> 8;               // 24 bits
    const uint32_t low8 = top & 0xffu;      // the next bits: 0x80 is one half
    const bool above = low8 > 0x80u || (low8 == 0x80u && rest != 0);
    const bool tie = low8 == 0x80u && rest == 0;
    mant += (above || (tie && (mant & 1u))) ? 1u : 0u;
    int ex = e;
    if (mant == (1u << 24)) {
        mant >>= 1;
        ++ex;
    }
    return fxp_bits_float(((uint32_t)(ex + 127) << 23) | (mant & 0x7fffffu));
}

}  // namespace erp

#undef ERP_FXP_FN
