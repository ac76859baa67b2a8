"""Generate tsr_math_tables.h: the lookup tables of the table-driven FP64
logarithm and exponential used by tsr_math.h.

Method: P. T. P. Tang, "Table-driven implementation of the exponential
function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989, and
"Table-driven implementation of the logarithm function in IEEE
floating-point arithmetic", ACM TOMS 16(4), 1990.  The tables hold
mathematical constants evaluated here in 200-bit arithmetic (mpmath) and
rounded to nearest double (hi) plus the rounded remainder (lo), so the
header is identical on every host and device that includes it.

Run:  python twoscalerich_gb300/csrc/gen_math_tables.py > twoscalerich_gb300/csrc/tsr_math_tables.h
"""
import mpmath

mpmath.mp.prec = 200
BITS = 8
N = 1 << BITS


def hexd(x):
    return float(x).hex()


def split(x):
    hi = float(x)
    lo = float(x - mpmath.mpf(hi))
    return hi, lo


def main():
    out = []
    out.append("/* Generated by gen_math_tables.py -- do not edit. */")
    out.append("#ifndef TSR_MATH_TABLES_H")
    out.append("#define TSR_MATH_TABLES_H")
    out.append("#define TSR_TBL_BITS %d" % BITS)
    out.append("#define TSR_TBL_N %d" % N)
    ln2 = mpmath.log(2)
    h, l = split(ln2)
    out.append("#define TSR_LN2_HI %s" % hexd(h))
    out.append("#define TSR_LN2_LO %s" % hexd(l))
    h, l = split(ln2 / N)
    out.append("#define TSR_LN2_N_HI %s  /* ln2 / %d */" % (hexd(h), N))
    out.append("#define TSR_LN2_N_LO %s" % hexd(l))
    out.append("#define TSR_N_LN2 %s  /* %d / ln2 */" % (hexd(N / ln2), N))
    out.append("#define TSR_INV_LN10 %s  /* 1 / ln10 */" % hexd(1 / mpmath.log(10)))
    # log table: c_i = 1 + i/N, entries {1/c_i, log(c_i) hi, log(c_i) lo, 0}
    out.append("/* {1/c_i, log(c_i) hi, log(c_i) lo, 0} with c_i = 1 + i/%d */" % N)
    out.append("#define TSR_LOG_TABLE_INIT { \\")
    for i in range(N):
        c = 1 + mpmath.mpf(i) / N
        inv = float(1 / c)
        hi, lo = split(mpmath.log(c))
        out.append("  {%s, %s, %s, 0.0}, \\" % (hexd(inv), hexd(hi), hexd(lo)))
    out.append("}")
    out.append("/* {2^(j/%d) hi, lo} */" % N)
    out.append("#define TSR_EXP_TABLE_INIT { \\")
    for j in range(N):
        hi, lo = split(mpmath.power(2, mpmath.mpf(j) / N))
        out.append("  {%s, %s}, \\" % (hexd(hi), hexd(lo)))
    out.append("}")
    out.append("#endif")
    print("\n".join(out))


if __name__ == "__main__":
    main()
