/*
 * tsr_math.h -- table-driven FP64 elementary functions shared, operation for
 * operation, by the sm_103a kernels and by every host-side evaluation of the
 * two-scale right-hand side.
 *
 * Why a private libm: the finite-difference Jacobian-vector product
 * Jv = (G(u + eps v) - G(u)) / eps divides any last-bit difference in G by
 * eps (~1e-8 relative), so two G implementations agree to 1e-12 in Jv only
 * if they agree bit for bit in G.  Bitwise agreement needs the same log/exp
 * on host and device, and the same sequence of IEEE operations around them.
 * Everything here is built from +, -, *, fma and integer bit manipulation
 * only; no host or device math library call is involved, and the code is
 * compiled without floating-point contraction on both sides.
 *
 * Methods (published): P. T. P. Tang, "Table-driven implementation of the
 * exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2),
 * 1989 (reduction x = (k/256) ln2 + r, 2^(j/256) table, polynomial in r);
 * P. T. P. Tang, "Table-driven implementation of the logarithm function in
 * IEEE floating-point arithmetic", ACM TOMS 16(4), 1990 (breakpoints
 * c_i = 1 + i/256, log(x) = E ln2 + log(c_i) + log1p((m - c_i)/c_i)).
 * The polynomials are the Taylor series of log1p and expm1 truncated where
 * the remainder falls below 2^-58 on the reduced interval.
 *
 * FP64 operation counts (the unit that bounds the kernels on GB300):
 *   tsr_log 14, tsr_log1p 18, tsr_exp 11, tsr_expm1 12.
 *
 * Deliberate domain limits (documented, tested):
 *   tsr_exp(x)   = 0 for x <= -707 (true value < 1e-307), inf above 709.78.
 *   tsr_expm1(x) = -1 for x <= -707.
 *   tsr_log1p(t) is meant for t >= 0 (used with t = (alpha|h|)^n).
 */
#ifndef TSR_MATH_H
#define TSR_MATH_H

#include <stdint.h>
#include <string.h>
#include <math.h>
#include "tsr_math_tables.h"

#if defined(__CUDACC__)
#define TSR_HD static __host__ __device__ __forceinline__
#else
#define TSR_HD static inline
#endif

typedef struct { double invc, logc_hi, logc_lo, pad; } tsr_log_entry;
typedef struct { double hi, lo; } tsr_exp_entry;
typedef struct {
    tsr_log_entry lg[TSR_TBL_N];
    tsr_exp_entry ex[TSR_TBL_N];
} tsr_math_tables;

#define TSR_MATH_TABLES_INIT { TSR_LOG_TABLE_INIT, TSR_EXP_TABLE_INIT }

TSR_HD uint64_t tsr_d2u(double x)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

TSR_HD double tsr_u2d(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

#define TSR_SHIFTER 0x1.8p52            /* 1.5 * 2^52 */
#define TSR_SHIFTER_BITS 0x4338000000000000ull
#define TSR_ONE_BITS 0x3FF0000000000000ull
#define TSR_MANT_MASK 0x000FFFFFFFFFFFFFull
#define TSR_ABS_MASK 0x7FFFFFFFFFFFFFFFull
#define TSR_DBL_MIN_BITS 0x0010000000000000ull
#define TSR_INF_BITS 0x7FF0000000000000ull
#define TSR_EXP_FAST_LIMIT_BITS 0x4086180000000000ull  /* 707.0 */
#define TSR_EXP_OVERFLOW 0x1.62e42fefa39efp+9          /* 709.78271289338397 */

/* log(x + corr) for positive, normal, finite x, where corr is a correction
 * far below ulp(x) scale (the rounding error of x); use_corr selects it. */
TSR_HD double tsr_log_core(double x, double corr, int use_corr,
                           const tsr_math_tables* T)
{
    uint64_t b = tsr_d2u(x);
    int64_t E = (int64_t)(b >> 52) - 1023;
    unsigned i = (unsigned)(b >> 44) & 0xFFu;
    uint64_t mb = (b & TSR_MANT_MASK) | TSR_ONE_BITS;                /* [1,2) */
    /* x in [1 - 2^-9, 1): reduce against c = 1 (u = x - 1, exact) so the
     * result keeps its relative accuracy instead of cancelling -ln2 + log c. */
    if (b >= 0x3FEFF00000000000ull && b < TSR_ONE_BITS) {
        E = 0;
        i = 0;
        mb = b;
    }
    double m = tsr_u2d(mb);
    double c = tsr_u2d(TSR_ONE_BITS | ((uint64_t)i << 44));         /* 1+i/256 */
    double f = m - c;                                                /* exact */
    if (use_corr && E < 1023)
        f = fma(corr, tsr_u2d((uint64_t)(1023 - E) << 52), f);      /* corr*2^-E */
    const tsr_log_entry* e = &T->lg[i];
    double u = f * e->invc;                                          /* [0,2^-8) */
    /* log1p(u) = u + u^2 q(u), q = -1/2 + u/3 - u^2/4 + u^3/5 - u^4/6 + u^5/7 */
    double q = fma(u, 0x1.2492492492492p-3, -0x1.5555555555555p-3);
    q = fma(q, u, 0x1.999999999999ap-3);
    q = fma(q, u, -0.25);
    q = fma(q, u, 0x1.5555555555555p-2);
    q = fma(q, u, -0.5);
    double p = fma(u * u, q, u);
    double ed = tsr_u2d(TSR_SHIFTER_BITS + (uint64_t)E) - TSR_SHIFTER; /* (double)E */
    double hi = fma(ed, TSR_LN2_HI, e->logc_hi);
    double lo = fma(ed, TSR_LN2_LO, e->logc_lo);
    return hi + (lo + p);
}

/* Special operands of log: zero, negative, subnormal, inf, NaN. */
TSR_HD double tsr_log_special(double x, const tsr_math_tables* T)
{
    uint64_t b = tsr_d2u(x);
    if ((b & TSR_ABS_MASK) == 0) return -INFINITY;
    if (b >> 63) return tsr_u2d(0x7FF8000000000000ull);           /* NaN */
    if (b >= TSR_INF_BITS) return x + x;                           /* inf/NaN */
    /* subnormal: scale by 2^54 */
    return tsr_log_core(x * 0x1p54, 0.0, 0, T) - 54.0 * TSR_LN2_HI;
}

TSR_HD double tsr_log(double x, const tsr_math_tables* T)
{
    uint64_t b = tsr_d2u(x);
    if (b - TSR_DBL_MIN_BITS >= TSR_INF_BITS - TSR_DBL_MIN_BITS)
        return tsr_log_special(x, T);
    return tsr_log_core(x, 0.0, 0, T);
}

/* log1p(t) for t >= 0 given s = 1 + t already rounded by the caller (the
 * two-scale model reuses s).  The rounding error of s is recovered exactly
 * (Fast2Sum ordered by magnitude) and folded into the reduced argument. */
TSR_HD double tsr_log1p_s(double t, double s, const tsr_math_tables* T)
{
    if (tsr_d2u(s) >= TSR_INF_BITS) return s + s;
    double corr = (t > 1.0) ? (1.0 - (s - t)) : (t - (s - 1.0));
    return tsr_log_core(s, corr, 1, T);
}

TSR_HD double tsr_log1p(double t, const tsr_math_tables* T)
{
    return tsr_log1p_s(t, 1.0 + t, T);
}

/* Shared reduction of exp/expm1: x = (k/256) ln2 + r, |r| <= ln2/512;
 * returns p = expm1(r) and sets j = k mod 256, M = (k - j)/256. */
TSR_HD double tsr_exp_reduce(double x, unsigned* j, int64_t* M)
{
    double t = fma(x, TSR_N_LN2, TSR_SHIFTER);
    int64_t k = (int64_t)(tsr_d2u(t) - TSR_SHIFTER_BITS);
    double kd = t - TSR_SHIFTER;
    double r = fma(-kd, TSR_LN2_N_HI, x);
    r = fma(-kd, TSR_LN2_N_LO, r);
    *j = (unsigned)k & 0xFFu;
    *M = (k - (int64_t)*j) / 256;
    /* expm1(r) = r + r^2 (1/2 + r/6 + r^2/24 + r^3/120) */
    double q = fma(r, 0x1.1111111111111p-7, 0x1.5555555555555p-5);
    q = fma(q, r, 0x1.5555555555555p-3);
    q = fma(q, r, 0.5);
    return fma(r * r, q, r);
}

/* exp(x) for |x| < 707 (no operand checks). */
TSR_HD double tsr_exp_fast(double x, const tsr_math_tables* T)
{
    unsigned j;
    int64_t M;
    double p = tsr_exp_reduce(x, &j, &M);
    const tsr_exp_entry* e = &T->ex[j];
    double y = e->hi + fma(e->hi, p, e->lo);
    return tsr_u2d(tsr_d2u(y) + ((uint64_t)M << 52));
}

TSR_HD double tsr_exp_special(double x, const tsr_math_tables* T)
{
    if (x != x) return x + x;
    if (x > 0.0) {
        if (x > TSR_EXP_OVERFLOW) return INFINITY;
        double h = tsr_exp_fast(0.5 * x, T);
        return h * h;
    }
    return 0.0;
}

TSR_HD double tsr_exp(double x, const tsr_math_tables* T)
{
    if ((tsr_d2u(x) & TSR_ABS_MASK) >= TSR_EXP_FAST_LIMIT_BITS)
        return tsr_exp_special(x, T);
    return tsr_exp_fast(x, T);
}

TSR_HD double tsr_expm1(double x, const tsr_math_tables* T)
{
    if ((tsr_d2u(x) & TSR_ABS_MASK) >= TSR_EXP_FAST_LIMIT_BITS) {
        if (x != x) return x + x;
        if (x > 0.0) return tsr_exp_special(x, T);
        return -1.0;
    }
    unsigned j;
    int64_t M;
    double p = tsr_exp_reduce(x, &j, &M);
    const tsr_exp_entry* e = &T->ex[j];
    double s2 = tsr_u2d((uint64_t)(1023 + M) << 52);               /* 2^M */
    double a = e->hi * s2 - 1.0;
    double b = fma(e->hi, p, e->lo) * s2;
    return a + b;
}

#endif /* TSR_MATH_H */
