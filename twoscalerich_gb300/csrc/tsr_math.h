/*
 * tsr_math.h -- FP64 elementary functions and division evaluated on the
 * integer pipe, shared operation for operation by the sm_103a kernels and by
 * every host-side evaluation of the two-scale right-hand side.
 *
 * Why a private libm: the finite-difference Jacobian-vector product
 * Jv = (G(u + eps v) - G(u)) / eps divides any last-bit difference in G by
 * eps (~1e-8 relative), so two G implementations agree to 1e-12 in Jv only
 * if they agree bit for bit in G.  Bitwise agreement needs the same log/exp
 * on host and device, and the same sequence of operations around them.
 *
 * Why the integer pipe: on GB300 the FP64 pipe retires ~1.65 instructions
 * per clock per SM (0.50 Top/s measured) while the 32-bit integer pipe
 * retires ~64.  The two-scale G is bound by FP64 instruction count, and its
 * van Genuchten relations need five elementary functions per node.  Here
 * the argument reductions, the table look-ups, the Taylor polynomials and
 * the final rounding to a double all run as exact fixed-point integer
 * arithmetic (64x64 -> 128-bit products, 128-bit sums), so none of these
 * functions issues an FP64 instruction on its usual path.  Integer
 * arithmetic is exactly reproducible, so host and device agree bit for bit.
 *
 * Methods (published): P. T. P. Tang, "Table-driven implementation of the
 * exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2),
 * 1989 (x = (k/256) ln2 + r, 2^(j/256) table); P. T. P. Tang, "Table-driven
 * implementation of the logarithm function in IEEE floating-point
 * arithmetic", ACM TOMS 16(4), 1990 (c_i = 1 + i/256, log x = E ln2 +
 * log c_i + log1p(u), u = (m - c_i)/c_i).  The polynomials are Taylor
 * series truncated below 2^-62 on the reduced interval; E ln2 + log c_i +
 * log1p(u) is summed exactly in 128-bit fixed point and rounded once.
 * Division: Newton-Raphson reciprocal of the divisor's mantissa in 64-bit
 * fixed point from the 8-bit seed 1/c_i, quotient estimate, then the exact
 * integer remainder settles the last unit and the round-to-nearest-even
 * decision (D. E. Knuth, TAOCP vol. 2, 4.3.1; P. Markstein, "Computation of
 * elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
 * Dev. 34(1), 1990): the result is the correctly rounded IEEE quotient.
 *
 * FP64 instructions per call on the paths the two-scale model takes:
 * tsr_log 0 (1 near x = 1), tsr_log1p_unit 0, tsr_exp 0, tsr_expm1 0
 * (1 for |x| < 2^-8 and for x >= ln2), tsr_div 0.  Accuracy against glibc:
 * within 1 ulp (tested); tsr_div equals the IEEE quotient (tested).
 *
 * Deliberate domain limits (documented, tested):
 *   tsr_exp(x)   = 0 for x <= -707 (true value < 1e-307), inf above 709.78.
 *   tsr_expm1(x) = -1 for x <= -707.
 *   tsr_log1p(t) is for t >= 0 (used with t = (alpha|h|)^n).
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

typedef __int128 tsr_i128;
typedef unsigned __int128 tsr_u128;

typedef struct { uint64_t invc63; int64_t logc_hi42, logc_r69, pad; } tsr_log_entry;
typedef struct { uint64_t hi, lo; } tsr_exp_qentry;
typedef struct {
    tsr_log_entry lg[TSR_TBL_N];
    int64_t ex62[TSR_TBL_N];
    tsr_exp_qentry ex126[TSR_TBL_N];
} tsr_math_tables;

#define TSR_MATH_TABLES_INIT { TSR_LOG_TABLE_INIT, TSR_EXP_TABLE_INIT, TSR_EXP126_TABLE_INIT }

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

/* high 64 bits of the 128-bit product */
TSR_HD uint64_t tsr_umulhi(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

/* high 64 bits of the signed 128-bit product (floor of a*b / 2^64) */
TSR_HD int64_t tsr_smulhi(int64_t a, int64_t b)
{
#if defined(__CUDA_ARCH__)
    return __mul64hi(a, b);
#else
    return (int64_t)(((__int128)a * b) >> 64);
#endif
}

TSR_HD int tsr_clz64(uint64_t x)   /* x != 0 */
{
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

/* floor(v / 2^n) for signed v, 0 <= n < 64 */
TSR_HD int64_t tsr_sar(int64_t v, int n)
{
    return v >= 0 ? (int64_t)((uint64_t)v >> n) : (int64_t)~((~(uint64_t)v) >> n);
}

#define TSR_SIGN_BIT 0x8000000000000000ull
#define TSR_ONE_BITS 0x3FF0000000000000ull
#define TSR_MANT_MASK 0x000FFFFFFFFFFFFFull
#define TSR_ABS_MASK 0x7FFFFFFFFFFFFFFFull
#define TSR_DBL_MIN_BITS 0x0010000000000000ull
#define TSR_INF_BITS 0x7FF0000000000000ull
#define TSR_EXP_FAST_LIMIT_BITS 0x4086180000000000ull  /* 707.0 */
#define TSR_EXP_OVERFLOW 0x1.62e42fefa39efp+9          /* 709.78271289338397 */

/* Sign tests on the integer pipe.  For every non-NaN x they equal the
 * comparisons x < 0.0, x >= 0.0 and x > 0.0 (-0.0 counts as zero). */
TSR_HD int tsr_lt0(double x)
{
    uint64_t b = tsr_d2u(x);
    return (b >> 63) != 0 && (b << 1) != 0;
}

TSR_HD int tsr_ge0(double x)
{
    uint64_t b = tsr_d2u(x);
    return (b >> 63) == 0 || (b << 1) == 0;
}

TSR_HD int tsr_gt0(double x)
{
    uint64_t b = tsr_d2u(x);
    return (b >> 63) == 0 && b != 0;
}

/* -x and -|x| by flipping the sign bit */
TSR_HD double tsr_negate(double x) { return tsr_u2d(tsr_d2u(x) ^ TSR_SIGN_BIT); }
TSR_HD double tsr_negabs(double x) { return tsr_u2d(tsr_d2u(x) | TSR_SIGN_BIT); }

/* Round v * 2^-scale to the nearest double (ties to even).  The result
 * must be a normal double; v == 0 gives +0. */
TSR_HD double tsr_fix2d(int64_t v, int scale)
{
    if (v == 0) return 0.0;
    uint64_t sgn = v < 0 ? TSR_SIGN_BIT : 0ull;
    uint64_t a = v < 0 ? (uint64_t)0 - (uint64_t)v : (uint64_t)v;
    int msb = 63 - tsr_clz64(a);
    uint64_t mant;
    if (msb > 52) {
        int sh = msb - 52;
        uint64_t rem = a & ((1ull << sh) - 1);
        uint64_t half = 1ull << (sh - 1);
        mant = a >> sh;
        if (rem > half || (rem == half && (mant & 1ull))) mant += 1;
    } else {
        mant = a << (52 - msb);
    }
    int64_t eb = (int64_t)msb - scale + 1023;       /* biased exponent */
    return tsr_u2d(sgn | (((uint64_t)(eb - 1) << 52) + mant));
}

/* The same for a signed 128-bit v (|v| < 2^127). */
TSR_HD double tsr_fix2d_128(tsr_i128 v, int scale)
{
    if (v == 0) return 0.0;
    uint64_t sgn = v < 0 ? TSR_SIGN_BIT : 0ull;
    tsr_u128 a = v < 0 ? (tsr_u128)0 - (tsr_u128)v : (tsr_u128)v;
    uint64_t hi = (uint64_t)(a >> 64);
    int msb = hi ? 127 - tsr_clz64(hi) : 63 - tsr_clz64((uint64_t)a);
    uint64_t mant;
    if (msb > 52) {
        int sh = msb - 52;
        tsr_u128 rem = a & (((tsr_u128)1 << sh) - 1);
        tsr_u128 half = (tsr_u128)1 << (sh - 1);
        mant = (uint64_t)(a >> sh);
        if (rem > half || (rem == half && (mant & 1ull))) mant += 1;
    } else {
        mant = (uint64_t)a << (52 - msb);
    }
    int64_t eb = (int64_t)msb - scale + 1023;
    return tsr_u2d(sgn | (((uint64_t)(eb - 1) << 52) + mant));
}

/* trunc(r * 2^scale) as a signed integer; |r| * 2^scale must be < 2^62 */
TSR_HD int64_t tsr_d2fix(double r, int scale)
{
    uint64_t b = tsr_d2u(r);
    int e = (int)((b >> 52) & 0x7FF);
    if (e == 0) return 0;
    uint64_t m = (b & TSR_MANT_MASK) | (1ull << 52);
    int sh = e - 1075 + scale;
    uint64_t a;
    if (sh >= 0) a = m << sh;
    else if (sh > -64) a = m >> (-sh);
    else a = 0;
    return (b >> 63) ? -(int64_t)a : (int64_t)a;
}

/* Q(u) = log1p(u)/u = 1 - u/2 + u^2/3 - ... - u^6/6 + u^7/7, |u| < 2^-8,
 * u given at scale 2^64; result at scale 2^62 */
TSR_HD int64_t tsr_log1p_q(int64_t U64)
{
    int64_t q = TSR_LOG1P_Q7;
    q = TSR_LOG1P_Q6 + tsr_smulhi(U64, q);
    q = TSR_LOG1P_Q5 + tsr_smulhi(U64, q);
    q = TSR_LOG1P_Q4 + tsr_smulhi(U64, q);
    q = TSR_LOG1P_Q3 + tsr_smulhi(U64, q);
    q = TSR_LOG1P_Q2 + tsr_smulhi(U64, q);
    return TSR_LOG1P_Q1 + tsr_smulhi(U64, q);
}

/* log1p(u) for an exact double u, 0 < |u| < 2^-8, with relative accuracy:
 * the exact mantissa of u times Q(u) in integer arithmetic. */
TSR_HD double tsr_log1p_small(double u)
{
    uint64_t b = tsr_d2u(u);
    int e = (int)((b >> 52) & 0x7FF);
    if (e == 0) return u;                               /* zero or subnormal */
    int64_t Q = tsr_log1p_q(tsr_d2fix(u, 64));
    uint64_t m = ((b & TSR_MANT_MASK) | (1ull << 52)) << 11;   /* leading bit 63 */
    int64_t P = (int64_t)tsr_umulhi(m, (uint64_t)Q);    /* |u| Q at scale 2^(1084 - e) */
    double r = tsr_fix2d(P, 1084 - e);
    return tsr_u2d(tsr_d2u(r) | (b & TSR_SIGN_BIT));
}

/* log(x + corr) for positive normal finite x away from 1 (x outside
 * [1 - 2^-9, 1 + 2^-8)); corr is a correction of the order of the rounding
 * error of x (use_corr selects it). */
TSR_HD double tsr_log_core(double x, double corr, int use_corr, const tsr_math_tables* T)
{
    uint64_t b = tsr_d2u(x);
    int64_t E = (int64_t)(b >> 52) - 1023;
    uint64_t mant = b & TSR_MANT_MASK;
    unsigned i = (unsigned)(mant >> 44);
    const tsr_log_entry* t = &T->lg[i];
    /* u = (m - c_i)/c_i at scale 2^71: (m - c_i) * 2^72 = low 44 bits << 20 */
    int64_t U71 = (int64_t)tsr_umulhi((mant & 0xFFFFFFFFFFFull) << 20, t->invc63);
    if (use_corr) {
        /* + corr 2^-E / c_i */
        int64_t C = tsr_d2fix(corr, (int)(71 - E));
        U71 += tsr_smulhi(C * 2, (int64_t)(t->invc63 >> 1)) * 2;
    }
    int64_t Q = tsr_log1p_q(tsr_sar(U71, 7));
    int64_t P69 = tsr_smulhi(U71, Q);                  /* log1p(u) at scale 2^69 */
    int64_t lo = P69 + t->logc_r69 + tsr_sar(E * TSR_LN2_R90, 21);
    int64_t K = E * TSR_LN2_HI42 + t->logc_hi42;        /* exact multiple of 2^-42 */
    /* K 2^-42 + lo 2^-69, summed exactly and rounded once */
    return tsr_fix2d_128((tsr_i128)K * ((tsr_i128)1 << 27) + lo, 69);
}

/* Special operands of log: zero, negative, subnormal, inf, NaN. */
TSR_HD double tsr_log(double x, const tsr_math_tables* T);

TSR_HD double tsr_log_special(double x, const tsr_math_tables* T)
{
    uint64_t b = tsr_d2u(x);
    if ((b & TSR_ABS_MASK) == 0) return -INFINITY;
    if (b >> 63) return tsr_u2d(0x7FF8000000000000ull);           /* NaN */
    if (b >= TSR_INF_BITS) return x + x;                           /* inf/NaN */
    /* subnormal: log(x 2^54) - 54 ln2, the scaled value is normal and away from 1 */
    return tsr_log_core(x * 0x1p54, 0.0, 0, T) - 54.0 * 0x1.62e42fefa39efp-1;
}

TSR_HD double tsr_log(double x, const tsr_math_tables* T)
{
    uint64_t b = tsr_d2u(x);
    if (b - TSR_DBL_MIN_BITS >= TSR_INF_BITS - TSR_DBL_MIN_BITS)
        return tsr_log_special(x, T);
    /* [1 - 2^-9, 1 + 2^-8): log1p of the exact x - 1 */
    if (b >= 0x3FEFF00000000000ull && b < 0x3FF0100000000000ull) {
        if (b == TSR_ONE_BITS) return 0.0;
        return tsr_log1p_small(x - 1.0);
    }
    return tsr_log_core(x, 0.0, 0, T);
}

/* log1p(e) for 0 <= e <= 1, also returning s1 = 1 + e rounded to double.
 * The sum 1 + e is formed exactly in fixed point and rounded once (scale
 * 2^112 for e >= 2^-60; below that 1 + e rounds to 1), so s1 costs no FP64
 * instruction; for e >= 2^-8 the exact sum is also the reduced argument of
 * the logarithm, so no correction term is needed. */
TSR_HD double tsr_log1p_unit(double e, double* s1, const tsr_math_tables* T)
{
    uint64_t b = tsr_d2u(e);
    if (b < 0x3F70000000000000ull) {                  /* e < 2^-8 */
        int ee = (int)(b >> 52);
        if (ee >= 963) {                               /* e >= 2^-60 */
            tsr_i128 S = ((tsr_i128)1 << 112) +
                         ((tsr_i128)((b & TSR_MANT_MASK) | (1ull << 52)) << (ee - 963));
            *s1 = tsr_fix2d_128(S, 112);
        } else {
            *s1 = 1.0;
        }
        if ((b << 1) == 0) return e;
        return tsr_log1p_small(e);
    }
    int ee = (int)(b >> 52);                           /* 1015 .. 1023 */
    uint64_t S = (1ull << 60) + (((b & TSR_MANT_MASK) | (1ull << 52)) << (ee - 1015));
    *s1 = tsr_fix2d((int64_t)S, 60);
    if (S == (1ull << 61)) return TSR_LN2_D;           /* e = 1 */
    /* S in (1, 2): c_i from the 8 bits below the leading one */
    unsigned i = (unsigned)(S >> 52) & 0xFFu;
    const tsr_log_entry* t = &T->lg[i];
    uint64_t F = S & ((1ull << 52) - 1);               /* (S - c_i) * 2^60 */
    int64_t U71 = (int64_t)tsr_umulhi(F << 12, t->invc63);
    int64_t Q = tsr_log1p_q(tsr_sar(U71, 7));
    int64_t lo = tsr_smulhi(U71, Q) + t->logc_r69;
    return tsr_fix2d_128((tsr_i128)t->logc_hi42 * ((tsr_i128)1 << 27) + lo, 69);
}

/* log1p(t) for t >= 0 given s = 1 + t already rounded by the caller.  For
 * t >= 2^-8 the rounding error of s is recovered (Fast2Sum ordered by
 * magnitude) and folded into the reduced argument; below, log1p(t) =
 * t Q(t) directly. */
TSR_HD double tsr_log1p_s(double t, double s, const tsr_math_tables* T)
{
    if (tsr_d2u(t) < 0x3F70000000000000ull) {          /* 0 <= t < 2^-8 */
        if (t == 0.0) return t;
        return tsr_log1p_small(t);
    }
    if (tsr_d2u(s) >= TSR_INF_BITS) return s + s;
    double corr = (t > 1.0) ? (1.0 - (s - t)) : (t - (s - 1.0));
    return tsr_log_core(s, corr, 1, T);
}

TSR_HD double tsr_log1p(double t, const tsr_math_tables* T)
{
    return tsr_log1p_s(t, 1.0 + t, T);
}

/* Shared argument reduction of exp/expm1, all on the integer pipe:
 * x = (k/256) ln2 + r with k = round(x 256/ln2) and |r| <= ln2/512 (plus
 * rounding of k).  For |x| >= 2^-14, x 2^66 is an exact 128-bit integer and
 * k ln2/256 is formed from ln2/256 at scale 2^106, so r66 = r 2^66 carries
 * r exactly but for one unit of 2^-66 (truncation of k ln2/256 toward
 * zero); below, k = 0 and r66 = trunc(x 2^66).  Returns Q(r) = expm1(r)/r
 * at scale 2^62 and sets r66, j = k mod 256 and M = (k - j)/256. */
TSR_HD int64_t tsr_exp_reduce(double x, int64_t* r66_out, unsigned* j, int64_t* M)
{
    /* k = round(x 256/ln2): (53-bit mantissa << 11) times 256/ln2 * 2^54,
     * high word, shifted by the exponent (|x| < 707) */
    uint64_t b = tsr_d2u(x);
    int ex = (int)((b >> 52) & 0x7FF);
    int sh = 1076 - ex;
    uint64_t mant = (b & TSR_MANT_MASK) | (1ull << 52);
    uint64_t ka = 0;
    if (sh < 64) {
        uint64_t P = tsr_umulhi(mant << 11, TSR_N_LN2_FIX54);
        ka = (P + (1ull << (sh - 1))) >> sh;
    }
    const int neg = (int)(b >> 63);
    const int64_t k = neg ? -(int64_t)ka : (int64_t)ka;
    int64_t r66;
    if (ex >= 1009) {
        /* |x| 2^66 < 2^77 and |k| ln2/256 2^66, both by magnitude */
        const tsr_u128 X = (tsr_u128)mant << (ex - 1009);
        const tsr_u128 C = ((tsr_u128)TSR_LN2_N_FIX106_HI << 64) | TSR_LN2_N_FIX106_LO;
        const tsr_u128 KC = ((tsr_u128)ka * C) >> 40;
        const tsr_i128 d = (tsr_i128)X - (tsr_i128)KC;         /* |x| - |k| ln2/256, |d| < 2^57 */
        r66 = neg ? -(int64_t)d : (int64_t)d;
    } else {
        r66 = tsr_d2fix(x, 66);                                /* k == 0 */
    }
    *j = (unsigned)k & 0xFFu;
    *M = (k - (int64_t)*j) / 256;
    *r66_out = r66;
    /* Q(r) = 1 + r/2 + r^2/6 + r^3/24 + r^4/120 + r^5/720 */
    const int64_t R = tsr_sar(r66, 2);                         /* r 2^64 */
    int64_t q = TSR_EXPM1_Q6;
    q = TSR_EXPM1_Q5 + tsr_smulhi(R, q);
    q = TSR_EXPM1_Q4 + tsr_smulhi(R, q);
    q = TSR_EXPM1_Q3 + tsr_smulhi(R, q);
    q = TSR_EXPM1_Q2 + tsr_smulhi(R, q);
    q = TSR_EXPM1_Q1 + tsr_smulhi(R, q);
    return q;
}

/* exp(x) for |x| < 707 (no operand checks) */
TSR_HD double tsr_exp_fast(double x, const tsr_math_tables* T)
{
    int64_t r66, M;
    unsigned j;
    int64_t q = tsr_exp_reduce(x, &r66, &j, &M);
    int64_t p = tsr_smulhi(r66, q);                     /* expm1(r) at scale 2^64 */
    int64_t Tj = T->ex62[j];
    int64_t y = Tj + tsr_smulhi(Tj, p);                 /* 2^(j/256) e^r at scale 2^62 */
    return tsr_fix2d(y, (int)(62 - M));
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
    if ((tsr_d2u(x) & TSR_ABS_MASK) < 0x3F70000000000000ull) {
        /* |x| < 2^-8: expm1(x) = x Q(x) without reduction */
        if ((tsr_d2u(x) << 1) == 0) return x;
        int64_t R = tsr_d2fix(x, 64);
        int64_t q = TSR_EXPM1_Q7;
        q = TSR_EXPM1_Q6 + tsr_smulhi(R, q);
        q = TSR_EXPM1_Q5 + tsr_smulhi(R, q);
        q = TSR_EXPM1_Q4 + tsr_smulhi(R, q);
        q = TSR_EXPM1_Q3 + tsr_smulhi(R, q);
        q = TSR_EXPM1_Q2 + tsr_smulhi(R, q);
        q = TSR_EXPM1_Q1 + tsr_smulhi(R, q);
        return x * tsr_fix2d(q, 62);
    }
    int64_t r66, M;
    unsigned j;
    int64_t q = tsr_exp_reduce(x, &r66, &j, &M);
    int64_t p = tsr_smulhi(r66, q);                     /* expm1(r) at scale 2^64 */
    if (M == 0 || M == -1) {
        /* the result cancels against 1: 2^(j/256) e^r - 1 in 128-bit fixed
         * point from the table entry at scale 2^126, rounded once */
        const tsr_exp_qentry* e = &T->ex126[j];
        const uint64_t pa = p < 0 ? (uint64_t)0 - (uint64_t)p : (uint64_t)p;
        const tsr_u128 mag = (tsr_u128)e->hi * pa + (((tsr_u128)e->lo * pa) >> 64);
        const tsr_i128 Tj = (tsr_i128)(((tsr_u128)e->hi << 64) | e->lo);   /* < 2^127 */
        const tsr_i128 y = p < 0 ? Tj - (tsr_i128)mag : Tj + (tsr_i128)mag;
        if (M == 0) return tsr_fix2d_128(y - ((tsr_i128)1 << 126), 126);
        /* y/2 - 1 at scale 2^127 (2^127 itself does not fit a signed 128-bit integer) */
        return tsr_fix2d_128((y - ((tsr_i128)1 << 126)) - ((tsr_i128)1 << 126), 127);
    }
    int64_t Tj = T->ex62[j];
    int64_t y = Tj + tsr_smulhi(Tj, p);                 /* scale 2^62 */
    if (M < 0) {
        /* y 2^M - 1 in fixed point (M <= -2: the result lies in (-1, -0.6)) */
        const int64_t ys = -M < 63 ? (y >> -M) : 0;
        return tsr_fix2d(ys - ((int64_t)1 << 62), 62);
    }
    return tsr_fix2d(y, (int)(62 - M)) - 1.0;
}

/* a / b, correctly rounded to nearest even, on the integer pipe for finite
 * a and normal b whose quotient is a normal double or zero; other operands
 * take the FP64 division (same result).  Reciprocal of b's mantissa d in
 * [1, 2): seed 1/c_i (8 bits, the logarithm table), three Newton steps
 * r <- r + r (1 - d r) in 64-bit fixed point (8 -> 16 -> 32 -> ~62 bits),
 * quotient estimate from a's mantissa times r, exact remainder correction
 * and rounding on the remainder. */
TSR_HD double tsr_div(double a, double b, const tsr_math_tables* T)
{
    const uint64_t ua = tsr_d2u(a), ub = tsr_d2u(b);
    const int ea = (int)((ua >> 52) & 0x7FF), eb = (int)((ub >> 52) & 0x7FF);
    if (eb == 0 || eb == 0x7FF || ea == 0x7FF) return a / b;
    const uint64_t sgn = (ua ^ ub) & TSR_SIGN_BIT;
    if (ea == 0) {
        if ((ua << 1) != 0) return a / b;                   /* subnormal a */
        return tsr_u2d(sgn);                                /* signed zero */
    }
    const uint64_t ma = (ua & TSR_MANT_MASK) | (1ull << 52);
    const uint64_t mb = (ub & TSR_MANT_MASK) | (1ull << 52);
    const int ge = ma >= mb;
    int E = ea - eb + (ge ? 1023 : 1022);
    uint64_t Q;
    if (mb == (1ull << 52)) {
        Q = ma;                                             /* b a power of two: exact */
        E = ea - eb + 1023;
    } else {
        /* r = 1/d at scale 2^64 (d > 1, so r < 1) */
        const unsigned i = (unsigned)((ub >> 44) & 0xFFu);
        uint64_t r = (i == 0) ? ~0ull : (T->lg[i].invc63 << 1);
        const uint64_t D = mb << 11;                        /* d at scale 2^63 */
        for (int it = 0; it < 3; ++it) {
            const uint64_t P = tsr_umulhi(D, r);            /* d r at scale 2^63 */
            if (P <= (1ull << 63)) r += tsr_umulhi(r, (1ull << 63) - P) << 1;
            else r -= tsr_umulhi(r, P - (1ull << 63)) << 1;
        }
        /* quotient mantissa: ma 2^s / mb, s = 52 (ma >= mb) or 53 */
        const int s = ge ? 52 : 53;
        const uint64_t est = tsr_umulhi(ma << 11, r);       /* ~ ma 2^63 / mb */
        Q = est >> (ge ? 11 : 10);
        /* remainder ma 2^s - Q mb; exact value small, formed modulo 2^64 */
        uint64_t rem = (ma << s) - Q * mb;
        for (int it = 0; it < 3 && (int64_t)rem < 0; ++it) {
            rem += mb;
            Q -= 1;
        }
        for (int it = 0; it < 3 && rem >= mb; ++it) {
            rem -= mb;
            Q += 1;
        }
        const uint64_t twice = rem << 1;
        if (twice > mb || (twice == mb && (Q & 1ull))) Q += 1;
        if (Q == (1ull << 53)) {
            Q = 1ull << 52;
            E += 1;
        }
    }
    if (E < 1 || E > 2046) return a / b;                    /* subnormal or overflow */
    return tsr_u2d(sgn | (((uint64_t)(E - 1) << 52) + Q));
}

#endif /* TSR_MATH_H */
