// tmath.h -- the oracle's exp, expm1, tanh, log and pow, written in plain IEEE double
// arithmetic, by the same published methods as the GPU library (so that host and device
// evaluations round identically: no libm, no fused multiply-add).  Methods:
//   exp:   Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2, with ln2 split into a 32-bit head
//          and a tail; exp(r) by its Taylor series to degree 13 (truncation < 1e-17); 2^k by ldexp.
//   expm1: Taylor series to degree 17 for |x| <= 1/2 (truncation < 1e-21), exp(x) - 1 beyond.
//   tanh:  -expm1(-2|x|) / (expm1(-2|x|) + 2) with the sign of x, 1 for |x| > 22.
//   log:   x = m 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s), s = (m-1)/(m+1),
//          atanh by its odd series to s^25 (|s| <= 0.1716); e ln2 with the split constant.
//   pow:   exp(y log x) for x > 0.
//   atan:  argument reduction to |t| <= tan(pi/8), then the Taylor series (atan_ below).
// Their accuracy against the platform libm is checked in the test-suite (a few ulp).
#pragma once
#include <math.h>

#if 0
#define TM_HD __host__ __device__
#else
#define TM_HD
#endif

namespace otm {

constexpr double LN2_HI = 0.6931471806019545;        // ln 2 rounded to 32 significant bits
constexpr double LN2_LO = -4.2009150726810846e-11;   // ln 2 - LN2_HI
constexpr double INV_LN2 = 1.4426950408889634;
constexpr double SQRT_HALF = 0.7071067811865476;

TM_HD inline double exp_(double x) {
    if (x != x) return x;
    if (x > 709.78) return HUGE_VAL;
    if (x < -745.2) return 0.0;
    double k = rint(x * INV_LN2);
    double r = (x - k * LN2_HI) - k * LN2_LO;
    double p = 1.0 / 6227020800.0;                     // 1/13!
    p = p * r + 1.0 / 479001600.0;
    p = p * r + 1.0 / 39916800.0;
    p = p * r + 1.0 / 3628800.0;
    p = p * r + 1.0 / 362880.0;
    p = p * r + 1.0 / 40320.0;
    p = p * r + 1.0 / 5040.0;
    p = p * r + 1.0 / 720.0;
    p = p * r + 1.0 / 120.0;
    p = p * r + 1.0 / 24.0;
    p = p * r + 1.0 / 6.0;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    return ldexp(p, (int)k);
}

TM_HD inline double expm1_(double x) {
    if (!(fabs(x) <= 0.5)) return x != x ? x : exp_(x) - 1.0;
    double p = 1.0 / 355687428096000.0;                // 1/17!
    p = p * x + 1.0 / 20922789888000.0;
    p = p * x + 1.0 / 1307674368000.0;
    p = p * x + 1.0 / 87178291200.0;
    p = p * x + 1.0 / 6227020800.0;
    p = p * x + 1.0 / 479001600.0;
    p = p * x + 1.0 / 39916800.0;
    p = p * x + 1.0 / 3628800.0;
    p = p * x + 1.0 / 362880.0;
    p = p * x + 1.0 / 40320.0;
    p = p * x + 1.0 / 5040.0;
    p = p * x + 1.0 / 720.0;
    p = p * x + 1.0 / 120.0;
    p = p * x + 1.0 / 24.0;
    p = p * x + 1.0 / 6.0;
    p = p * x + 0.5;
    p = p * x + 1.0;
    return p * x;
}

TM_HD inline double tanh_(double x) {
    if (x != x) return x;
    double ax = fabs(x);
    double t;
    if (ax > 22.0) t = 1.0;
    else {
        double e = expm1_(-2.0 * ax);
        t = -e / (e + 2.0);
    }
    return copysign(t, x);
}

TM_HD inline double log_(double x) {
    if (x != x || x < 0.0) return NAN;
    if (x == 0.0) return -HUGE_VAL;
    if (x == HUGE_VAL) return x;
    int e;
    double m = frexp(x, &e);
    if (m < SQRT_HALF) { m = m * 2.0; e = e - 1; }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s;
    double p = 1.0 / 25.0;
    p = p * s2 + 1.0 / 23.0;
    p = p * s2 + 1.0 / 21.0;
    p = p * s2 + 1.0 / 19.0;
    p = p * s2 + 1.0 / 17.0;
    p = p * s2 + 1.0 / 15.0;
    p = p * s2 + 1.0 / 13.0;
    p = p * s2 + 1.0 / 11.0;
    p = p * s2 + 1.0 / 9.0;
    p = p * s2 + 1.0 / 7.0;
    p = p * s2 + 1.0 / 5.0;
    p = p * s2 + 1.0 / 3.0;
    p = p * s2 + 1.0;
    double lm = 2.0 * s * p;
    double de = (double)e;
    return de * LN2_HI + (de * LN2_LO + lm);
}

TM_HD inline double pow_(double x, double y) { return exp_(y * log_(x)); }

// atan: |x| > 1 by pi/2 - atan(1/|x|); t > tan(pi/8) by pi/4 + atan((t-1)/(t+1)); then the
// Taylor series t - t^3/3 + t^5/5 - ... to t^43/43 (|t| <= tan(pi/8): truncation < 1e-18);
// the sign of x restored
TM_HD inline double atan_(double x) {
    if (x != x) return x;
    const double PI_2 = 1.5707963267948966, PI_4 = 0.7853981633974483;
    const double TAN_PI_8 = 0.41421356237309503;
    double ax = fabs(x);
    bool inv = ax > 1.0;
    double t = inv ? 1.0 / ax : ax;
    bool red = t > TAN_PI_8;
    if (red) t = (t - 1.0) / (t + 1.0);
    double z = -(t * t);
    double p = 1.0 / 43.0;
    p = p * z + 1.0 / 41.0;
    p = p * z + 1.0 / 39.0;
    p = p * z + 1.0 / 37.0;
    p = p * z + 1.0 / 35.0;
    p = p * z + 1.0 / 33.0;
    p = p * z + 1.0 / 31.0;
    p = p * z + 1.0 / 29.0;
    p = p * z + 1.0 / 27.0;
    p = p * z + 1.0 / 25.0;
    p = p * z + 1.0 / 23.0;
    p = p * z + 1.0 / 21.0;
    p = p * z + 1.0 / 19.0;
    p = p * z + 1.0 / 17.0;
    p = p * z + 1.0 / 15.0;
    p = p * z + 1.0 / 13.0;
    p = p * z + 1.0 / 11.0;
    p = p * z + 1.0 / 9.0;
    p = p * z + 1.0 / 7.0;
    p = p * z + 1.0 / 5.0;
    p = p * z + 1.0 / 3.0;
    p = p * z + 1.0 / 1.0;
    double r = t * p;
    if (red) r = PI_4 + r;
    if (inv) r = PI_2 - r;
    return copysign(r, x);
}

}  // namespace otm
