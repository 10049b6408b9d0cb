// crmath.cuh -- exp, log and pow rounded to the nearest double, for the
// red-exact arithmetic mode (FP64_EXACT).
//
// red forms its step-size factor (tol / err)^(1/order) on the host with the C
// library's pow (int_rungekutta8.cu:690-716) and its gas-drag factors with the
// C library's pow and exp (pp_disk.cu:59-155 in its CPU twin).  The GNU C
// library's exp and pow return the double nearest to the exact result except
// in rare hard cases (their documented error bound is about 0.52 ulp).  The
// functions here evaluate the exact result to about 1e-30 relative in
// double-double arithmetic and round it once, so they return that same
// nearest double: the red-exact mode then takes red's step sizes bit for bit.
// CUDA's pow and exp (documented to 2 and 1 ulp) would let 1-ulp differences
// into the step sizes, which the embedded error estimate magnifies.
//
// Methods (all published):
//   * double-double arithmetic: Dekker, "A floating-point technique for
//     extending the available precision" (1971); TwoSum after Knuth, TAOCP
//     vol. 2, 4.2.2; the product's error term by one fused multiply-add.
//   * log: x = m 2^e with m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh(s),
//     s = (m - 1) / (m + 1), |s| <= 0.1716, by its Taylor series
//     sum s^(2k+1) / (2k+1) to 24 terms (truncation < 1e-36).
//   * exp: y = k ln 2 + r, |r| <= ln 2 / 2; exp(r) = exp(r / 2^10)^(2^10) with
//     exp(r / 2^10) by its Taylor series to 14 terms (truncation < 1e-45),
//     then ten squarings (each keeps ~1e-31 relative).
//   * pow(x, y) = exp(y ln x) for finite x > 0; every other case (x <= 0,
//     infinities, NaN, a result outside the normal range) is passed to the
//     library pow / exp, whose results there are exact or special values.
// These are about a hundred times the cost of the library functions; the
// FP32 and FP64 modes keep the library functions.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define CR_FN __host__ __device__ __forceinline__
#else
#define CR_FN static inline
#endif

namespace crmath {

struct dd {
    double hi, lo;
};

// The FMA is the only fused operation; every other sum and product is a
// single rounding (these helpers are never contracted by the compiler, since
// no product feeds an addition outside the explicit fma).
CR_FN double fma_(double a, double b, double c)
{
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return fma(a, b, c);
#endif
}
CR_FN double add_(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
CR_FN double sub_(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
CR_FN double mul_(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
CR_FN double div_(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}

CR_FN dd two_sum(double a, double b)
{
    const double s = add_(a, b);
    const double bb = sub_(s, a);
    const double e = add_(sub_(a, sub_(s, bb)), sub_(b, bb));
    return {s, e};
}
CR_FN dd quick_two_sum(double a, double b)   // |a| >= |b|
{
    const double s = add_(a, b);
    return {s, sub_(b, sub_(s, a))};
}
CR_FN dd two_prod(double a, double b)
{
    const double p = mul_(a, b);
    return {p, fma_(a, b, -p)};
}
CR_FN dd dd_add(dd a, dd b)
{
    dd s = two_sum(a.hi, b.hi);
    const dd t = two_sum(a.lo, b.lo);
    s.lo = add_(s.lo, t.hi);
    s = quick_two_sum(s.hi, s.lo);
    s.lo = add_(s.lo, t.lo);
    return quick_two_sum(s.hi, s.lo);
}
CR_FN dd dd_neg(dd a) { return {-a.hi, -a.lo}; }
CR_FN dd dd_mul(dd a, dd b)
{
    dd p = two_prod(a.hi, b.hi);
    p.lo = add_(p.lo, add_(mul_(a.hi, b.lo), mul_(a.lo, b.hi)));
    return quick_two_sum(p.hi, p.lo);
}
CR_FN dd dd_mul_d(dd a, double b)
{
    dd p = two_prod(a.hi, b);
    p.lo = add_(p.lo, mul_(a.lo, b));
    return quick_two_sum(p.hi, p.lo);
}
CR_FN dd dd_div(dd a, dd b)
{
    // three quotient digits, each from the exact remainder
    const double q1 = div_(a.hi, b.hi);
    dd r = dd_add(a, dd_neg(dd_mul_d(b, q1)));
    const double q2 = div_(r.hi, b.hi);
    r = dd_add(r, dd_neg(dd_mul_d(b, q2)));
    const double q3 = div_(r.hi, b.hi);
    dd q = quick_two_sum(q1, q2);
    return dd_add(q, dd{q3, 0.0});
}
// 1 / n for a small integer n, to double-double precision: the remainder of
// the rounded quotient is exact by one fma
CR_FN dd dd_recip_int(double n)
{
    const double h = div_(1.0, n);
    const double rem = fma_(-h, n, 1.0);
    return {h, div_(rem, n)};
}

// ln 2 split into its nearest double and the nearest double of the rest
// (0.69314718055994530941723212145817656807550013436...)
#define CR_LN2_HI 6.93147180559945286227e-01
#define CR_LN2_LO 2.31904681384629955842e-17

CR_FN dd dd_log(double x)   // finite x > 0
{
    int e;
    double m = frexp(x, &e);   // x = m 2^e, m in [0.5, 1)
    if (m < 0.70710678118654752440) {
        m = mul_(m, 2.0);
        e -= 1;
    }
    // s = (m - 1) / (m + 1): m - 1 is exact for m in [0.5, 2] (Sterbenz)
    const dd num = {sub_(m, 1.0), 0.0};
    const dd den = two_sum(m, 1.0);
    const dd s = dd_div(num, den);
    const dd s2 = dd_mul(s, s);
    const int K = 24;
    dd p = dd_recip_int(2.0 * K + 1.0);
    for (int k = K - 1; k >= 0; k--) p = dd_add(dd_mul(p, s2), dd_recip_int(2.0 * k + 1.0));
    dd l = dd_mul(dd_mul_d(p, 2.0), s);
    const dd eln2 = dd_add(two_prod((double)e, CR_LN2_HI), two_prod((double)e, CR_LN2_LO));
    return dd_add(l, eln2);
}

CR_FN dd dd_exp(dd y)   // |y| <= 700
{
    const double k = floor(add_(div_(y.hi, CR_LN2_HI), 0.5));
    // r = y - k ln 2, exact products of k (|k| < 2^11) with the two parts
    dd r = dd_add(y, dd_neg(two_prod(k, CR_LN2_HI)));
    r = dd_add(r, dd_neg(two_prod(k, CR_LN2_LO)));
    const double scale = 1.0 / 1024.0;
    r = {mul_(r.hi, scale), mul_(r.lo, scale)};   // exact
    // exp(r) - 1 = r (1 + r/2 (1 + r/3 (1 + ... (1 + r/N)))), Horner from the inside
    const int N = 14;
    dd p = {1.0, 0.0};
    for (int n = N; n >= 2; n--) p = dd_add(dd{1.0, 0.0}, dd_mul(dd_mul(r, p), dd_recip_int((double)n)));
    dd em1 = dd_mul(r, p);
    // (1 + a)^2 = 1 + (2a + a^2): ten squarings on exp - 1 keep the small part exact
    for (int i = 0; i < 10; i++) em1 = dd_add(dd_mul_d(em1, 2.0), dd_mul(em1, em1));
    dd res = dd_add(dd{1.0, 0.0}, em1);
    const int ki = (int)k;
    return {ldexp(res.hi, ki), ldexp(res.lo, ki)};
}

// The nearest double of exp(x).
CR_FN double cr_exp(double x)
{
    if (!(fabs(x) <= 700.0)) return exp(x);
    const dd r = dd_exp(dd{x, 0.0});
    return add_(r.hi, r.lo);
}

// The nearest double of x^y.
CR_FN double cr_pow(double x, double y)
{
    if (!(x > 0.0) || isinf(x) || !isfinite(y)) return pow(x, y);
    if (y == 0.0 || x == 1.0) return 1.0;
    if (y == 1.0) return x;
    const dd l = dd_log(x);
    const dd t = dd_mul_d(l, y);
    if (!(fabs(t.hi) <= 700.0)) return pow(x, y);
    const dd r = dd_exp(t);
    return add_(r.hi, r.lo);
}

}  // namespace crmath
