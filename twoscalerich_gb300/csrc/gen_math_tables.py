"""Generate tsr_math_tables.h: the lookup tables of the table-driven FP64
logarithm and exponential of tsr_math.h.

Method: P. T. P. Tang, "Table-driven implementation of the exponential
function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989, and
"Table-driven implementation of the logarithm function in IEEE
floating-point arithmetic", ACM TOMS 16(4), 1990 -- breakpoints c_i =
1 + i/256 for the logarithm and 2^(j/256) for the exponential.  The entries
are mathematical constants evaluated here in 200-bit arithmetic (mpmath)
and stored as fixed-point integers, so the header is identical on every host
and device that includes it:

  log:  1/c_i * 2^63 (unsigned), log(c_i) split into a multiple of 2^-42
        (stored as the integer log(c_i) * 2^42) and the remainder * 2^69;
  exp:  2^(j/256) * 2^62, and 2^(j/256) * 2^126 as two 64-bit words (used
        where expm1 cancels against 1); ln2/256 * 2^106 as two 64-bit words
        (the fixed-point argument reduction).

Run:  python gen_math_tables.py > tsr_math_tables.h
"""
import mpmath

mpmath.mp.prec = 200
BITS = 8
N = 1 << BITS


def rnd(x):
    return int(mpmath.nint(x))


def main():
    out = []
    out.append("/* Generated by gen_math_tables.py -- do not edit. */")
    out.append("#ifndef TSR_MATH_TABLES_H")
    out.append("#define TSR_MATH_TABLES_H")
    out.append("#define TSR_TBL_BITS %d" % BITS)
    out.append("#define TSR_TBL_N %d" % N)
    ln2 = mpmath.log(2)
    out.append("#define TSR_LN2_N_HI %s  /* ln2 / %d, high part */" % (float(ln2 / N).hex(), N))
    out.append("#define TSR_LN2_N_LO %s" % float(ln2 / N - mpmath.mpf(float(ln2 / N))).hex())
    out.append("#define TSR_N_LN2 %s  /* %d / ln2 */" % (float(N / ln2).hex(), N))
    out.append("#define TSR_INV_LN10 %s  /* 1 / ln10 */" % float(1 / mpmath.log(10)).hex())
    out.append("#define TSR_LN2_D %s  /* ln2 rounded to double */" % float(ln2).hex())
    out.append("#define TSR_N_LN2_FIX54 %dULL  /* %d / ln2 * 2^54 */" % (rnd(N / ln2 * 2 ** 54), N))
    c106 = rnd(ln2 / N * 2 ** 106)
    out.append("#define TSR_LN2_N_FIX106_HI %dULL  /* ln2 / %d * 2^106, bits 64..127 */" % (c106 >> 64, N))
    out.append("#define TSR_LN2_N_FIX106_LO %dULL  /* bits 0..63 */" % (c106 & (2 ** 64 - 1)))
    l42 = rnd(ln2 * 2 ** 42)
    out.append("#define TSR_LN2_HI42 %dLL  /* ln2 * 2^42, rounded */" % l42)
    out.append("#define TSR_LN2_R90 %dLL  /* (ln2 - TSR_LN2_HI42 * 2^-42) * 2^90 */"
               % rnd((ln2 - mpmath.mpf(l42) / 2 ** 42) * 2 ** 90))
    # fixed-point Taylor coefficients
    for k in range(1, 9):
        out.append("#define TSR_LOG1P_Q%d %dLL  /* (-1)^(k+1)/k * 2^62 */"
                   % (k, rnd(mpmath.mpf((-1) ** (k + 1)) / k * 2 ** 62)))
    for k in range(1, 8):
        out.append("#define TSR_EXPM1_Q%d %dLL  /* 1/k! * 2^62 */"
                   % (k, rnd(mpmath.mpf(1) / mpmath.factorial(k) * 2 ** 62)))
    out.append("/* {2^63/c_i, log(c_i)*2^42 rounded, remainder*2^69, 0}, c_i = 1 + i/%d */" % N)
    out.append("#define TSR_LOG_TABLE_INIT { \\")
    for i in range(N):
        c = 1 + mpmath.mpf(i) / N
        inv = rnd(2 ** 63 / c)
        hi = rnd(mpmath.log(c) * 2 ** 42)
        r = rnd((mpmath.log(c) - mpmath.mpf(hi) / 2 ** 42) * 2 ** 69)
        out.append("  {%dULL, %dLL, %dLL, 0LL}, \\" % (inv, hi, r))
    out.append("}")
    out.append("/* 2^(j/%d) * 2^62 */" % N)
    out.append("#define TSR_EXP_TABLE_INIT { \\")
    for j in range(N):
        out.append("  %dLL, \\" % rnd(mpmath.power(2, mpmath.mpf(j) / N) * 2 ** 62))
    out.append("}")
    out.append("/* 2^(j/%d) * 2^126 rounded: {bits 64..127, bits 0..63} */" % N)
    out.append("#define TSR_EXP126_TABLE_INIT { \\")
    for j in range(N):
        v = rnd(mpmath.power(2, mpmath.mpf(j) / N) * 2 ** 126)
        out.append("  {%dULL, %dULL}, \\" % (v >> 64, v & (2 ** 64 - 1)))
    out.append("}")
    out.append("#endif")
    print("\n".join(out))


if __name__ == "__main__":
    main()
