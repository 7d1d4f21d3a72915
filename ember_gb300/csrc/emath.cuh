// Exponential and logarithm in FP64 for the kinetics kernels, written for
// this library from textbook methods so that the device code and the CPU
// restatement can evaluate them with the same operation sequence:
//   exp: Cody-Waite reduction x = k ln2 + r with a two-part ln2 applied by
//        FMA, |r| <= ln2/2, then the degree-13 Taylor polynomial of e^r in
//        Horner form (truncation error < 4e-18 relative), scaled by 2^k
//        through the exponent bits.
//   log: x = 2^e m with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s),
//        s = (m-1)/(m+1), |s| < 0.1716, series to s^21 (truncation < 1e-19).
// Polynomial coefficients are the reciprocal factorials 1/n! and 2/(2k+1)
// rounded to the nearest double; ln2 is split into its nearest double and
// the nearest double of the remainder. Both functions are accurate to about
// 1-2 ulp against the C library's exp/log (checked on the CPU restatement,
// which runs the same operation sequence); on the GPU they give the CPU
// restatement's bits, which every chemistry parity test exercises.
#pragma once

#include <cstdint>

namespace ember {

#define EMATH_LN2_HI 0.6931471805599453
#define EMATH_LN2_LO 2.3190468138462996e-17
#define EMATH_LOG2E 1.4426950408889634
#define EMATH_SQRT2_BITS 0x3ff6a09e667f3bcdLL  // 1.4142135623730951, the double nearest sqrt 2
#define EMATH_LN10 2.302585092994046
#define EMATH_LOG10E 0.4342944819032518

__device__ __forceinline__ double em_pow2i(int k) {
    return __longlong_as_double(static_cast<long long>(k + 1023) << 52);
}

// |x| <= 708 as a test of the magnitude bits on the integer pipe: inside it
// none of em_exp's range cases applies, so the FP64 compares run only
// outside it, with the same results.
#define EMATH_EXP_PLAIN_BITS 0x4086200000000000LL  // 708.0

__device__ __forceinline__ double em_exp(double x) {
    if ((__double_as_longlong(x) & 0x7fffffffffffffffLL) > EMATH_EXP_PLAIN_BITS) {
        if (x != x) return x;
        if (x > 709.782712893384) return __longlong_as_double(0x7ff0000000000000LL);
        if (x < -745.1332191019412) return 0.0;
    }
    const double kd = rint(x * EMATH_LOG2E);
    double r = fma(-kd, EMATH_LN2_HI, x);
    r = fma(-kd, EMATH_LN2_LO, r);
    double p = 1.6059043836821613e-10;
    p = fma(p, r, 2.08767569878681e-09);
    p = fma(p, r, 2.505210838544172e-08);
    p = fma(p, r, 2.755731922398589e-07);
    p = fma(p, r, 2.7557319223985893e-06);
    p = fma(p, r, 2.48015873015873e-05);
    p = fma(p, r, 0.0001984126984126984);
    p = fma(p, r, 0.001388888888888889);
    p = fma(p, r, 0.008333333333333333);
    p = fma(p, r, 0.041666666666666664);
    p = fma(p, r, 0.16666666666666666);
    p = fma(p, r, 0.5);
    p = fma(p, r, 1.0);
    p = fma(p, r, 1.0);
    int k = static_cast<int>(kd);
    if (k > 1023) return (p * em_pow2i(1023)) * em_pow2i(k - 1023);
    if (k < -1022) return (p * em_pow2i(k + 1000)) * em_pow2i(-1000);
    return p * em_pow2i(k);
}

__device__ __forceinline__ double em_log(double x) {
    long long bits = __double_as_longlong(x);
    // positive and finite exactly when 0 < bits < the bits of +inf; the
    // special cases (zero, negative, NaN, +inf) are tested only outside
    if (bits <= 0 || bits >= 0x7ff0000000000000LL) {
        if (!(x > 0.0)) return x == 0.0 ? __longlong_as_double(0xfff0000000000000LL) : __longlong_as_double(0x7ff8000000000000LL);
        return x;  // +inf
    }
    int e = 0;
    if (bits < 0x0010000000000000LL) {  // subnormal: scale by 2^54
        x *= 18014398509481984.0;
        bits = __double_as_longlong(x);
        e = -54;
    }
    e += static_cast<int>((bits >> 52) & 0x7ff) - 1023;
    // m in [1, 2); above sqrt 2 it is halved (exactly: the exponent field
    // drops by one). Positive doubles order as their bit patterns, so the
    // comparison with sqrt 2 runs on the integer pipe.
    long long mb = (bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL;
    if (mb > EMATH_SQRT2_BITS) {
        mb -= 0x0010000000000000LL;
        e += 1;
    }
    const double m = __longlong_as_double(mb);
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double q = 0.09523809523809523;
    q = fma(q, s2, 0.10526315789473684);
    q = fma(q, s2, 0.11764705882352941);
    q = fma(q, s2, 0.13333333333333333);
    q = fma(q, s2, 0.15384615384615385);
    q = fma(q, s2, 0.18181818181818182);
    q = fma(q, s2, 0.2222222222222222);
    q = fma(q, s2, 0.2857142857142857);
    q = fma(q, s2, 0.4);
    q = fma(q, s2, 0.6666666666666666);
    const double t = fma(s, s2 * q, 2.0 * s);
    const double ed = static_cast<double>(e);
    return fma(ed, EMATH_LN2_HI, fma(ed, EMATH_LN2_LO, t));
}

__device__ __forceinline__ double em_log10(double x) { return em_log(x) * EMATH_LOG10E; }
__device__ __forceinline__ double em_exp10(double x) { return em_exp(x * EMATH_LN10); }

}  // namespace ember
