// Exact binary32 <-> binary64 conversions on the integer pipes.
//
// GB300 executes FP64 instructions, conversions between FP32 and FP64
// included, at about two per clock per SM; the FP32-bulk kernels convert every
// residual sum to FP64 and every state component back to FP32 each stage, so
// they do it with integer operations instead, straight from the IEEE 754
// encodings: the results equal the hardware conversions (round to nearest
// even for double -> float, exact for float -> double), including signed
// zeros, subnormals, infinities and NaNs (quiet bit and payload kept).
#pragma once

#include <cstdint>

namespace lfm {
namespace dev {

// The general conversions (every class of input).
__device__ __forceinline__ double f32_to_f64_any(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    const unsigned ex = (u >> 23) & 0xffu;
    const unsigned man = u & 0x7fffffu;
    unsigned long long bits;
    if (ex - 1u < 254u) {                       // normal: rebias 127 -> 1023
        bits = sign | ((unsigned long long)(ex + 896u) << 52) | ((unsigned long long)man << 29);
    } else if (ex == 255u) {                    // infinity, NaN
        bits = sign | (0x7ffULL << 52) | ((unsigned long long)man << 29);
    } else if (man == 0u) {                     // zero
        bits = sign;
    } else {                                    // subnormal: man * 2^-149, renormalised
        const int k = 31 - __clz((int)man);     // leading one of the 23-bit field
        bits = sign | ((unsigned long long)(k + 874) << 52) |
               ((unsigned long long)(man ^ (1u << k)) << (52 - k));
    }
    return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ float f64_to_f32_any(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int ex = (int)((b >> 52) & 0x7ffu);
    const unsigned long long man = b & 0xfffffffffffffULL;
    if (ex == 0x7ff) {                          // infinity, NaN (quiet bit set on NaN)
        const unsigned m = man ? (0x400000u | (unsigned)(man >> 29)) : 0u;
        return __uint_as_float(sign | 0x7f800000u | m);
    }
    const int e = ex - 896;                     // binary32 biased exponent
    if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
    unsigned long long sig;                     // significand with the hidden bit
    int shift;                                  // right shift to the 23-bit field
    if (e > 0) {
        sig = man | (1ULL << 52);
        shift = 29;
    } else {                                    // binary32 subnormal or zero
        if (ex == 0 || e < -24) return __uint_as_float(sign);
        sig = man | (1ULL << 52);
        shift = 30 - e;
    }
    unsigned long long q = sig >> shift;
    const unsigned long long rem = sig & ((1ULL << shift) - 1);
    const unsigned long long half = 1ULL << (shift - 1);
    if (rem > half || (rem == half && (q & 1ULL))) ++q;   // round to nearest even
    unsigned r;
    if (e > 0) {
        // q holds 1.m with the hidden bit at 2^23; a carry to 2^24 bumps the exponent
        const unsigned hi = (unsigned)(q >> 23);          // 1 or 2
        const int en = e + (int)hi - 1;
        if (en >= 255) return __uint_as_float(sign | 0x7f800000u);
        r = ((unsigned)en << 23) | ((unsigned)q & 0x7fffffu);
        if (hi == 2) r = ((unsigned)en << 23) | (((unsigned)(q >> 1)) & 0x7fffffu);
    } else {
        r = (unsigned)q;                        // may round up into the smallest normal
    }
    return __uint_as_float(sign | r);
}

// Fast paths on 32-bit words for the common classes, the general code for
// the rest.
//
// float -> double, normal x: the 11-bit exponent is the 8-bit one + 896 and
// the 52-bit fraction the 23-bit one followed by 29 zeros, so the high word
// is sign | ((x & 0x7fffffff) >> 3) + (896 << 20) and the low word x << 29;
// zeros keep only the sign.
__device__ __forceinline__ double f32_to_f64(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned mag = u & 0x7fffffffu;
    if (mag - 0x00800000u < 0x7f000000u)        // normal: exponent field 1 .. 254
        return __hiloint2double((int)((u & 0x80000000u) | ((mag >> 3) + 0x38000000u)), (int)(u << 29));
    if (mag == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return f32_to_f64_any(x);
}

// double -> float with a normal result before rounding (double exponent
// field 897 .. 1150, binary32 exponent 1 .. 254): the top 31 bits below the
// sign of (exponent - 896, 23 fraction bits) are one funnel shift of the high
// and low words minus 896 << 23 (mod 2^32); the 29 dropped fraction bits
// round to nearest even by adding 0x0fffffff plus the kept lowest bit and
// carrying bit 29 in. A carry out of the fraction raises the exponent, and out
// of exponent 254 gives the infinity that rounding to nearest produces.
__device__ __forceinline__ float f64_to_f32(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned ex = (hi >> 20) & 0x7ffu;
    if (ex - 897u < 254u) {
        const unsigned r = __funnelshift_l(lo, hi, 3) - 0xc0000000u;
        const unsigned up = ((lo & 0x1fffffffu) + (r & 1u) + 0x0fffffffu) >> 29;
        return __uint_as_float((hi & 0x80000000u) | (r + up));
    }
    if (((hi & 0x7fffffffu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
    return f64_to_f32_any(x);
}

}  // namespace dev
}  // namespace lfm
