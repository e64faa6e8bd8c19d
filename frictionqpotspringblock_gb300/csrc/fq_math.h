/*
 * Portable, deterministic elementary functions for the disorder transforms
 * (log / pow used by the weibull, exponential, power and pareto yield-distance
 * distributions) and for the Smooth potential (sin).
 *
 * Why this file exists: the reference computes these with the host libm
 * (prrng's distribution transforms call std::log / std::pow; the Smooth
 * potential calls std::sin, include/FrictionQPotSpringBlock/detail.h:406).
 * CUDA's libm and glibc's libm do not round identically, so a device that
 * called CUDA's `log` would drift from the CPU by an ulp now and then.  Every
 * function here is built only from correctly-rounded IEEE-754 primitives
 * (add, sub, mul, div, sqrt, fma) issued through explicit macros, so the very
 * same source gives bit-identical results on the host (gcc, -ffp-contract=off)
 * and on sm_103a (nvcc, `__dadd_rn`-style intrinsics that cannot be contracted).
 *
 * Method (textbook, no library internals): double-double arithmetic (Dekker /
 * Knuth two-sum and fma-based two-product); log by reduction to
 * m in [1/sqrt2, sqrt2] and the series 2*atanh((m-1)/(m+1)); exp by reduction
 * modulo ln2 and a Taylor series; sin by reduction modulo pi/2 and Taylor
 * series for sin / cos.  Constants are correctly rounded double-double
 * expansions of ln2, pi/2 and 1/k! .  Accuracy is well below one ulp
 * (the results are correctly rounded except in rare near-midpoint cases), so
 * they almost always agree with glibc bit for bit; the tests measure that.
 */
#ifndef FQSB_FQ_MATH_H
#define FQSB_FQ_MATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define FQ_HD __host__ __device__ __forceinline__
#if defined(__CUDA_ARCH__)
#define FQ_ADD(a, b) __dadd_rn((a), (b))
#define FQ_SUB(a, b) __dsub_rn((a), (b))
#define FQ_MUL(a, b) __dmul_rn((a), (b))
#define FQ_DIV(a, b) __ddiv_rn((a), (b))
#define FQ_FMA(a, b, c) __fma_rn((a), (b), (c))
#define FQ_SQRT(a) __dsqrt_rn(a)
#else
#include <math.h>
#define FQ_ADD(a, b) ((a) + (b))
#define FQ_SUB(a, b) ((a) - (b))
#define FQ_MUL(a, b) ((a) * (b))
#define FQ_DIV(a, b) ((a) / (b))
#define FQ_FMA(a, b, c) fma((a), (b), (c))
#define FQ_SQRT(a) sqrt(a)
#endif
#else
#include <math.h>
#include <string.h>
#define FQ_HD static inline
/* Host build: must be compiled with -ffp-contract=off (the oracle's recipe does so). */
#define FQ_ADD(a, b) ((a) + (b))
#define FQ_SUB(a, b) ((a) - (b))
#define FQ_MUL(a, b) ((a) * (b))
#define FQ_DIV(a, b) ((a) / (b))
#define FQ_FMA(a, b, c) fma((a), (b), (c))
#define FQ_SQRT(a) sqrt(a)
#endif

FQ_HD uint64_t fq_bits(double x)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, sizeof(b));
    return b;
#endif
}

FQ_HD double fq_from_bits(uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, sizeof(x));
    return x;
#endif
}

typedef struct {
    double hi;
    double lo;
} fq_dd;

FQ_HD fq_dd fq_dd_make(double hi, double lo)
{
    fq_dd r;
    r.hi = hi;
    r.lo = lo;
    return r;
}

/* Exact a + b = s + e (Knuth). */
FQ_HD fq_dd fq_two_sum(double a, double b)
{
    double s = FQ_ADD(a, b);
    double bb = FQ_SUB(s, a);
    double e = FQ_ADD(FQ_SUB(a, FQ_SUB(s, bb)), FQ_SUB(b, bb));
    return fq_dd_make(s, e);
}

/* Exact a + b = s + e when |a| >= |b| (Dekker). */
FQ_HD fq_dd fq_fast_two_sum(double a, double b)
{
    double s = FQ_ADD(a, b);
    double e = FQ_SUB(b, FQ_SUB(s, a));
    return fq_dd_make(s, e);
}

/* Exact a * b = p + e using one fma. */
FQ_HD fq_dd fq_two_prod(double a, double b)
{
    double p = FQ_MUL(a, b);
    double e = FQ_FMA(a, b, -p);
    return fq_dd_make(p, e);
}

FQ_HD fq_dd fq_dd_add(fq_dd x, fq_dd y)
{
    fq_dd s = fq_two_sum(x.hi, y.hi);
    fq_dd t = fq_two_sum(x.lo, y.lo);
    double e = FQ_ADD(s.lo, t.hi);
    fq_dd u = fq_fast_two_sum(s.hi, e);
    e = FQ_ADD(u.lo, t.lo);
    return fq_fast_two_sum(u.hi, e);
}

FQ_HD fq_dd fq_dd_neg(fq_dd x)
{
    return fq_dd_make(-x.hi, -x.lo);
}

FQ_HD fq_dd fq_dd_mul(fq_dd x, fq_dd y)
{
    fq_dd p = fq_two_prod(x.hi, y.hi);
    double c = FQ_ADD(FQ_MUL(x.hi, y.lo), FQ_MUL(x.lo, y.hi));
    double e = FQ_ADD(p.lo, c);
    return fq_fast_two_sum(p.hi, e);
}

FQ_HD fq_dd fq_dd_mul_d(fq_dd x, double d)
{
    fq_dd p = fq_two_prod(x.hi, d);
    double e = FQ_ADD(p.lo, FQ_MUL(x.lo, d));
    return fq_fast_two_sum(p.hi, e);
}

/* ln 2, pi/2, 1/3, 1/5 as correctly rounded double-double expansions. */
#define FQ_LN2_HI 0x1.62e42fefa39efp-1
#define FQ_LN2_LO 0x1.abc9e3b39803fp-56
#define FQ_INV_LN2 0x1.71547652b82fep+0
#define FQ_PIO2_HI 0x1.921fb54442d18p+0
#define FQ_PIO2_LO 0x1.1a62633145c07p-54
#define FQ_TWO_OVER_PI 0x1.45f306dc9c883p-1
#define FQ_THIRD_HI 0x1.5555555555555p-2
#define FQ_THIRD_LO 0x1.5555555555555p-56
#define FQ_FIFTH_HI 0x1.999999999999ap-3
#define FQ_FIFTH_LO -0x1.999999999999ap-57

#define FQ_NAN_BITS 0x7ff8000000000000ULL
#define FQ_INF_BITS 0x7ff0000000000000ULL

/* log(m) for m in [1/sqrt2, sqrt2], as a double-double. */
FQ_HD fq_dd fq_log_core(double m)
{
    double f = FQ_SUB(m, 1.0); /* exact (Sterbenz) */
    if (f == 0.0) {
        return fq_dd_make(0.0, 0.0);
    }
    /* s = f / (2 + f) in double-double */
    fq_dd d = fq_two_sum(2.0, f);
    double s_hi = FQ_DIV(f, d.hi);
    double r = FQ_FMA(-s_hi, d.hi, f);
    r = FQ_FMA(-s_hi, d.lo, r);
    double s_lo = FQ_DIV(r, d.hi);
    fq_dd S = fq_fast_two_sum(s_hi, s_lo);
    fq_dd T = fq_dd_mul(S, S); /* t = s^2 <= 0.0295 */
    double t = T.hi;
    /* w = 1/7 + t/9 + t^2/11 + ... + t^12/31 (plain double Horner) */
    double w = 1.0 / 31.0;
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 29.0);
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 27.0);
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 25.0);
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 23.0);
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 21.0);
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 19.0);
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 17.0);
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 15.0);
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 13.0);
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 11.0);
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 9.0);
    w = FQ_ADD(FQ_MUL(w, t), 1.0 / 7.0);
    /* A = 1/5 + t*w ; B = 1/3 + t*A ; C = t*B ; log m = 2 (s + s C) */
    fq_dd A = fq_dd_add(fq_dd_make(FQ_FIFTH_HI, FQ_FIFTH_LO), fq_dd_mul_d(T, w));
    fq_dd B = fq_dd_add(fq_dd_make(FQ_THIRD_HI, FQ_THIRD_LO), fq_dd_mul(T, A));
    fq_dd C = fq_dd_mul(T, B);
    fq_dd R = fq_dd_add(S, fq_dd_mul(S, C));
    return fq_dd_make(FQ_MUL(R.hi, 2.0), FQ_MUL(R.lo, 2.0));
}

/* log(x) as a double-double, for finite x > 0. */
FQ_HD fq_dd fq_log_dd(double x)
{
    uint64_t b = fq_bits(x);
    int e_adj = 0;
    if ((b >> 52) == 0) { /* subnormal */
        x = FQ_MUL(x, 0x1p54);
        b = fq_bits(x);
        e_adj = -54;
    }
    int e = (int)((b >> 52) & 0x7ff) - 1023 + e_adj;
    uint64_t mb = b & 0x000fffffffffffffULL;
    double m;
    if (mb > 0x6a09e667f3bcdULL) {
        m = fq_from_bits(mb | 0x3fe0000000000000ULL);
        e += 1;
    }
    else {
        m = fq_from_bits(mb | 0x3ff0000000000000ULL);
    }
    fq_dd L = fq_log_core(m);
    if (e != 0) {
        fq_dd E = fq_dd_mul_d(fq_dd_make(FQ_LN2_HI, FQ_LN2_LO), (double)e);
        L = fq_dd_add(E, L);
    }
    return L;
}

/* Natural logarithm. */
FQ_HD double fq_log(double x)
{
    if (x != x) {
        return x;
    }
    if (x < 0.0) {
        return fq_from_bits(FQ_NAN_BITS);
    }
    if (x == 0.0) {
        return -fq_from_bits(FQ_INF_BITS);
    }
    if (fq_bits(x) == FQ_INF_BITS) {
        return x;
    }
    fq_dd L = fq_log_dd(x);
    return FQ_ADD(L.hi, L.lo);
}

/* 1/k! for k = 0..20 as double-double (hi, lo). */
#define FQ_NFACT 21
#if defined(__CUDACC__)
__host__ __device__
#endif
static inline void fq_inv_factorial(int k, double* hi, double* lo)
{
    /* values computed in high precision and rounded to double-double */
    switch (k) {
        case 0: *hi = 1.0; *lo = 0.0; break;
        case 1: *hi = 1.0; *lo = 0.0; break;
        case 2: *hi = 0.5; *lo = 0.0; break;
        case 3: *hi = 0x1.5555555555555p-3; *lo = 0x1.5555555555555p-57; break;
        case 4: *hi = 0x1.5555555555555p-5; *lo = 0x1.5555555555555p-59; break;
        case 5: *hi = 0x1.1111111111111p-7; *lo = 0x1.1111111111111p-63; break;
        case 6: *hi = 0x1.6c16c16c16c17p-10; *lo = -0x1.f49f49f49f49fp-65; break;
        case 7: *hi = 0x1.a01a01a01a01ap-13; *lo = 0x1.a01a01a01a01ap-73; break;
        case 8: *hi = 0x1.a01a01a01a01ap-16; *lo = 0x1.a01a01a01a01ap-76; break;
        case 9: *hi = 0x1.71de3a556c734p-19; *lo = -0x1.c154f8ddc6c00p-73; break;
        case 10: *hi = 0x1.27e4fb7789f5cp-22; *lo = 0x1.cbbc05b4fa99ap-76; break;
        case 11: *hi = 0x1.ae64567f544e4p-26; *lo = -0x1.c062e06d1f209p-80; break;
        case 12: *hi = 0x1.1eed8eff8d898p-29; *lo = -0x1.2aec959e14c06p-83; break;
        case 13: *hi = 0x1.6124613a86d09p-33; *lo = 0x1.f28e0cc748ebep-87; break;
        case 14: *hi = 0x1.93974a8c07c9dp-37; *lo = 0x1.05d6f8a2efd1fp-92; break;
        case 15: *hi = 0x1.ae7f3e733b81fp-41; *lo = 0x1.1d8656b0ee8cbp-97; break;
        case 16: *hi = 0x1.ae7f3e733b81fp-45; *lo = 0x1.1d8656b0ee8cbp-101; break;
        case 17: *hi = 0x1.952c77030ad4ap-49; *lo = 0x1.ac981465ddc6cp-103; break;
        case 18: *hi = 0x1.6827863b97d97p-53; *lo = 0x1.eec01221a8b0bp-107; break;
        case 19: *hi = 0x1.2f49b46814157p-57; *lo = 0x1.2650f61dbdcb4p-112; break;
        default: *hi = 0x1.e542ba4020225p-62; *lo = 0x1.ea72b4afe3c2fp-120; break;
    }
}

/* 2^n as a double for -1022 <= n <= 1023. */
FQ_HD double fq_pow2i(int n)
{
    return fq_from_bits((uint64_t)(n + 1023) << 52);
}

/* exp of a double-double argument, rounded to double. */
FQ_HD double fq_exp_dd(fq_dd P)
{
    if (P.hi != P.hi) {
        return P.hi;
    }
    if (P.hi > 709.8) {
        return fq_from_bits(FQ_INF_BITS);
    }
    if (P.hi < -745.2) {
        return 0.0;
    }
    double kf = FQ_MUL(P.hi, FQ_INV_LN2);
    int n = (int)(kf >= 0.0 ? FQ_ADD(kf, 0.5) : FQ_SUB(kf, 0.5));
    fq_dd r = fq_dd_add(P, fq_dd_neg(fq_dd_mul_d(fq_dd_make(FQ_LN2_HI, FQ_LN2_LO), (double)n)));
    /* Horner in double-double over 1/k!, k = 20..0 ; |r| <= 0.35 */
    double ch, cl;
    fq_inv_factorial(20, &ch, &cl);
    fq_dd p = fq_dd_make(ch, cl);
    for (int k = 19; k >= 0; --k) {
        fq_inv_factorial(k, &ch, &cl);
        p = fq_dd_add(fq_dd_mul(p, r), fq_dd_make(ch, cl));
    }
    double y = FQ_ADD(p.hi, p.lo);
    /* scale by 2^n in at most two exact steps (one rounding if the result is subnormal) */
    if (n > 1023) {
        y = FQ_MUL(y, fq_pow2i(1023));
        n -= 1023;
    }
    else if (n < -1022) {
        y = FQ_MUL(y, fq_pow2i(-1022));
        n += 1022;
        if (n < -1022) {
            return 0.0;
        }
    }
    return FQ_MUL(y, fq_pow2i(n));
}

/* exp(x). */
FQ_HD double fq_exp(double x)
{
    return fq_exp_dd(fq_dd_make(x, 0.0));
}

/* x^y for x >= 0 (the only case the yield-distance transforms need). */
FQ_HD double fq_pow(double x, double y)
{
    if (y == 1.0) {
        return x;
    }
    if (x != x || y != y) {
        return fq_from_bits(FQ_NAN_BITS);
    }
    if (y == 0.0 || x == 1.0) {
        return 1.0;
    }
    if (x < 0.0) {
        return fq_from_bits(FQ_NAN_BITS);
    }
    if (x == 0.0) {
        return y > 0.0 ? 0.0 : fq_from_bits(FQ_INF_BITS);
    }
    if (fq_bits(x) == FQ_INF_BITS) {
        return y > 0.0 ? x : 0.0;
    }
    if (y == 0.5) {
        return FQ_SQRT(x); /* correctly rounded, equal to the correctly rounded pow */
    }
    if (y == 2.0) {
        return FQ_MUL(x, x);
    }
    fq_dd L = fq_log_dd(x);
    return fq_exp_dd(fq_dd_mul_d(L, y));
}

/* sin(x + shift * pi/2) for shift in {0, 1}: reduction by pi/2 in double-double, Taylor series. */
FQ_HD double fq_sin_shift(double x, int shift)
{
    if (x != x) {
        return x;
    }
    if ((fq_bits(x) & 0x7fffffffffffffffULL) == FQ_INF_BITS) {
        return fq_from_bits(FQ_NAN_BITS);
    }
    if (x == 0.0 && shift == 0) {
        return x;
    }
    double kf = FQ_MUL(x, FQ_TWO_OVER_PI);
    double nf = kf >= 0.0 ? (double)(int64_t)FQ_ADD(kf, 0.5) : (double)(int64_t)FQ_SUB(kf, 0.5);
    int64_t n = (int64_t)nf;
    fq_dd r = fq_dd_add(fq_dd_make(x, 0.0), fq_dd_neg(fq_dd_mul_d(fq_dd_make(FQ_PIO2_HI, FQ_PIO2_LO), nf)));
    fq_dd r2 = fq_dd_mul(r, r);
    int q = (int)((n + shift) & 3);
    double ch, cl;
    fq_dd p;
    if (q == 0 || q == 2) {
        /* sin r = r * sum_{j} (-1)^j r^{2j} / (2j+1)!  (j = 0..9) */
        fq_inv_factorial(19, &ch, &cl);
        p = fq_dd_make(-ch, -cl);
        for (int j = 8; j >= 0; --j) {
            fq_inv_factorial(2 * j + 1, &ch, &cl);
            fq_dd c = (j & 1) ? fq_dd_make(-ch, -cl) : fq_dd_make(ch, cl);
            p = fq_dd_add(fq_dd_mul(p, r2), c);
        }
        p = fq_dd_mul(p, r);
    }
    else {
        /* cos r = sum_{j} (-1)^j r^{2j} / (2j)!  (j = 0..10) */
        fq_inv_factorial(20, &ch, &cl);
        p = fq_dd_make(ch, cl);
        for (int j = 9; j >= 0; --j) {
            fq_inv_factorial(2 * j, &ch, &cl);
            fq_dd c = (j & 1) ? fq_dd_make(-ch, -cl) : fq_dd_make(ch, cl);
            p = fq_dd_add(fq_dd_mul(p, r2), c);
        }
    }
    double y = FQ_ADD(p.hi, p.lo);
    return (q >= 2) ? -y : y;
}

/* sin(x). */
FQ_HD double fq_sin(double x)
{
    return fq_sin_shift(x, 0);
}

/* cos(x) = sin(x + pi/2), the quadrant shifted exactly (no rounding of x + pi/2). */
FQ_HD double fq_cos(double x)
{
    return fq_sin_shift(x, 1);
}

/* ---------------------------------------------------------------- erf / erfc / erfinv
 * For the normal quantile of thermal forcing, mean + stddev sqrt(2) erfinv(2 r - 1).
 *
 * erf near a grid point.  With x_i = i/64 and G_i = (2/sqrt(pi)) exp(-x_i^2),
 *     erf(x_i + h) = erf(x_i) + G_i S(h),  erfc(x_i + h) = erfc(x_i) - G_i S(h),
 *     S(h) = sum_k q_k h^(k+1),  q_k = p_k / (k+1),  sum_k p_k h^k = exp(-2 x_i h - h^2),
 * the Taylor series of erf's derivative about x_i (p_k = (-1)^k H_k(x_i) / k!).  erf(x_i), erfc(x_i),
 * G_i and q_0 .. q_15 come from a table (fq_erf_table.h, 60-digit mpmath; the leading coefficients as
 * double-doubles).  With |h| <= 1/128 the truncation error is below 1e-29 relative to G_i, so the
 * double-double sum resolves erfc(x) to ~1e-27 relative up to x = 6.
 *
 * erfinv(y): bracket |y| (or 1 - |y| > 1/2, which is exact, against erfc) in the table, interpolate
 * linearly (error <= 4e-4), then Halley steps x -= d / (1 + x d), d = residual / derivative: two with a
 * double residual (to ~1 ulp), the last with the double-double residual.  That last correction is about
 * an ulp and is computed to ~16 digits, so the result is the correctly rounded erfinv except within
 * ~1e-16 ulp of a rounding midpoint.  Host and device run the same code (the table is duplicated into
 * device memory), so they agree bit for bit.
 */
#include "fq_erf_table.h"

#if defined(__CUDACC__)
__device__ static const double fq_erf_tab_dev[FQ_ERF_N][FQ_ERF_ROW] = FQ_ERF_TABLE_INIT;
#endif
static const double fq_erf_tab_host[FQ_ERF_N][FQ_ERF_ROW] = FQ_ERF_TABLE_INIT;

/* row i of the erf table: erf (hi, lo), erfc (hi, lo), G (hi, lo), q_0 .. q_7 (hi, lo), q_8 .. q_15 */
FQ_HD const double* fq_erf_row(int i)
{
#if defined(__CUDA_ARCH__)
    return fq_erf_tab_dev[i];
#else
    return fq_erf_tab_host[i];
#endif
}

/* q_k of a row, rounded to double */
FQ_HD double fq_erf_q(const double* row, int k)
{
    return k < FQ_ERF_K_DD ? row[6 + 2 * k] : row[6 + 2 * FQ_ERF_K_DD + (k - FQ_ERF_K_DD)];
}

/* nearest grid point of x >= 0 */
FQ_HD int fq_erf_cell(double x)
{
    int i = (int)FQ_ADD(FQ_MUL(x, 64.0), 0.5);
    return i < FQ_ERF_N - 1 ? i : FQ_ERF_N - 1;
}

/* erfinv(y), -1 <= y <= 1. */
FQ_HD double fq_erfinv(double y)
{
    if (y != y) {
        return y;
    }
    const double a = y < 0.0 ? -y : y;
    if (a > 1.0) {
        return fq_from_bits(FQ_NAN_BITS);
    }
    if (a == 1.0) {
        return y < 0.0 ? -fq_from_bits(FQ_INF_BITS) : fq_from_bits(FQ_INF_BITS);
    }
    if (a == 0.0) {
        return y;
    }
    if (a < 0x1p-500) {
        /* erfinv(a) = a sqrt(pi)/2 (1 + pi a^2 / 12 + ...): the correction is below 2^-1000 */
        const double s = FQ_MUL(a, 0x1p+600);
        fq_dd pr = fq_two_prod(s, 0x1.c5bf891b4ef6bp-1);
        double x = FQ_ADD(pr.hi, FQ_ADD(pr.lo, FQ_MUL(s, -0x1.618f13eb7ca89p-55)));
        x = FQ_MUL(x, 0x1p-600);
        return y < 0.0 ? -x : x;
    }
    const int tail = a > 0.5;
    const double q = FQ_SUB(1.0, a); /* exact for a >= 1/2 */
    const double target = tail ? q : a;
    /* bracket: the last grid point with erf(x_i) <= a (erfc(x_i) >= q in the tail) */
    int lo = 0, hi = FQ_ERF_N - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        const double v = fq_erf_row(mid)[tail ? 2 : 0];
        if (tail ? v >= q : v <= a) {
            lo = mid;
        }
        else {
            hi = mid;
        }
    }
    const double f0 = fq_erf_row(lo)[tail ? 2 : 0];
    const double f1 = fq_erf_row(lo + 1)[tail ? 2 : 0];
    double t = FQ_DIV(FQ_SUB(target, f0), FQ_SUB(f1, f0));
    t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
    double x = FQ_MUL(FQ_ADD((double)lo, t), 0x1p-6);

    for (int it = 0; it < 3; ++it) {
        const int cell = fq_erf_cell(x);
        const double* row = fq_erf_row(cell);
        const double h = FQ_SUB(x, FQ_MUL((double)cell, 0x1p-6)); /* exact */
        double r;
        if (it < 2) {
            double s = fq_erf_q(row, FQ_ERF_K - 1);
            for (int k = FQ_ERF_K - 2; k >= 0; --k) {
                s = FQ_ADD(FQ_MUL(s, h), fq_erf_q(row, k));
            }
            const double gs = FQ_MUL(row[4], FQ_MUL(s, h));
            r = tail ? FQ_SUB(FQ_SUB(row[2], gs), q) : FQ_SUB(FQ_ADD(row[0], gs), a);
        }
        else {
            double s = fq_erf_q(row, FQ_ERF_K - 1);
            for (int k = FQ_ERF_K - 2; k >= FQ_ERF_K_DD; --k) {
                s = FQ_ADD(FQ_MUL(s, h), fq_erf_q(row, k));
            }
            fq_dd S = fq_dd_make(s, 0.0);
            for (int k = FQ_ERF_K_DD - 1; k >= 0; --k) {
                S = fq_dd_add(fq_dd_mul_d(S, h), fq_dd_make(row[6 + 2 * k], row[7 + 2 * k]));
            }
            const fq_dd gs = fq_dd_mul(fq_dd_make(row[4], row[5]), fq_dd_mul_d(S, h));
            const fq_dd v = tail ? fq_dd_add(fq_dd_make(row[2], row[3]), fq_dd_neg(gs))
                                 : fq_dd_add(fq_dd_make(row[0], row[1]), gs);
            r = FQ_ADD(FQ_SUB(v.hi, target), v.lo);
        }
        /* derivative (2/sqrt(pi)) exp(-x^2) = G sum_k (k+1) q_k h^k */
        double g = FQ_MUL((double)FQ_ERF_K, fq_erf_q(row, FQ_ERF_K - 1));
        for (int k = FQ_ERF_K - 2; k >= 0; --k) {
            g = FQ_ADD(FQ_MUL(g, h), FQ_MUL((double)(k + 1), fq_erf_q(row, k)));
        }
        const double deriv = FQ_MUL(row[4], g);
        const double d = tail ? FQ_DIV(-r, deriv) : FQ_DIV(r, deriv);
        x = FQ_SUB(x, FQ_DIV(d, FQ_ADD(1.0, FQ_MUL(x, d))));
    }
    return y < 0.0 ? -x : x;
}

#endif
