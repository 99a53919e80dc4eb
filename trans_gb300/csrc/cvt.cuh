// cvt.cuh -- double <-> float conversions on the integer pipe.
//
// On GB300 a hardware conversion between double and float (either direction) issues on the
// FP64 pipe, at the FP64 rate: 0.059 warp instructions per SM per clock, against 0.050 for
// a DFMA and 3.7 for an FFMA (measured), and an FP64 instruction costs the pipe the same time
// whatever the number of active lanes.  The mixed-precision kernels convert FP64 state to FP32
// and FP32 increments back for every cell, so those conversions, not their arithmetic, filled
// the FP64 pipe.  The versions below build the IEEE-754 result from the bit fields with integer
// operations, which run on the integer pipe and overlap the FP64 work; a round trip is 3.2x
// faster than the hardware pair.  No path issues an FP64 instruction: normal results and
// zeros are inline, the rare cases (subnormal results, overflow, infinities, NaN) are a call.
//
//   f32_rn(x): x rounded to the nearest float, ties to even -- bit-identical to (float)x
//     (a NaN stays a NaN, quiet).
//   f64_of(f): the exact double value of f -- bit-identical to (double)f (NaN stays NaN).
//
// Both are checked against the hardware conversions on random and edge-case bit patterns by
// trans_check_conversions.
#pragma once
#include <cuda_runtime.h>

namespace tg {

// subnormal and zero float results (rounded), overflow to infinity, infinities and NaN
static __device__ __noinline__ unsigned f32_rn_rare(unsigned long long u) {
    const unsigned hi = (unsigned)(u >> 32), e = (hi >> 20) & 0x7ffu;
    const unsigned sign = hi & 0x80000000u;
    if (e >= 1151u) {                                // |x| >= 2^128, infinity or NaN
        const bool nan = e == 2047u && (u & 0xfffffffffffffull) != 0ull;
        return sign | (nan ? 0x7fc00000u | (unsigned)((u & 0xfffffffffffffull) >> 29) : 0x7f800000u);
    }
    // |x| < 2^-126: the float subnormal sig * 2^(e - 1075) / 2^-149 = sig / 2^(926 - e), rounded
    // to nearest even (a carry into bit 23 gives the smallest normal float, as it should)
    const unsigned shift = 926u - e;                 // >= 30
    if (e == 0u || shift > 63u) return sign;         // below half the smallest subnormal
    const unsigned long long sig = (u & 0xfffffffffffffull) | 0x10000000000000ull;
    const unsigned long long q = sig >> shift, rem = sig & ((1ull << shift) - 1ull), half = 1ull << (shift - 1u);
    return sign | ((unsigned)q + ((rem > half || (rem == half && (q & 1ull))) ? 1u : 0u));
}

__device__ __forceinline__ float f32_rn(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
    const unsigned e = (hi >> 20) & 0x7ffu;          // biased double exponent
    if (e - 897u < 254u) {                           // float exponent 1..254: a normal float
        // exponent rebiased (1023 -> 127), the top 23 of 52 mantissa bits; the 29 dropped
        // bits round to nearest, ties to even (a carry runs into the exponent, as it should)
        unsigned r = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
        const unsigned rem = lo & 0x1fffffffu;
        r += (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ? 1u : 0u;
        return __uint_as_float((hi & 0x80000000u) | r);
    }
    if ((u << 1) == 0ull) return __uint_as_float(hi & 0x80000000u);    // +-0
    return __uint_as_float(f32_rn_rare(u));
}

// subnormal floats (normalised), infinities and NaN (quiet)
static __device__ __noinline__ unsigned long long f64_of_rare(unsigned v) {
    const unsigned long long sign = (unsigned long long)(v & 0x80000000u) << 32;
    const unsigned e = (v >> 23) & 0xffu, m = v & 0x7fffffu;
    if (e == 255u) return sign | 0x7ff0000000000000ull | ((unsigned long long)m << 29) | (m ? 0x8000000000000ull : 0ull);
    const int k = 31 - __clz(m);                     // m * 2^-149 = 1.f * 2^(k - 149), m != 0
    return sign | ((unsigned long long)(k + 874) << 52) | (((unsigned long long)m << (52 - k)) & 0xfffffffffffffull);
}

__device__ __forceinline__ double f64_of(float f) {
    const unsigned v = __float_as_uint(f);
    const unsigned e = (v >> 23) & 0xffu;
    if (e - 1u < 254u)                               // normal: rebias 127 -> 1023, widen the mantissa
        return __hiloint2double((int)((v & 0x80000000u) | ((e + 896u) << 20) | ((v >> 3) & 0xfffffu)), (int)(v << 29));
    if ((v << 1) == 0u) return __hiloint2double((int)(v & 0x80000000u), 0);  // +-0
    return __longlong_as_double((long long)f64_of_rare(v));
}

}  // namespace tg
