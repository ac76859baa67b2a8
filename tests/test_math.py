"""The library's FP64 elementary functions (tsr_math.h: integer-pipe
fixed-point Tang tables) against the C library, which is what a CPU
implementation of the reference would call.  Bound: 1 ulp."""
import math

import numpy as np
import pytest

import oracle


def ulps(a, b):
    if a == b:
        return 0.0
    return abs(a - b) / abs(math.ulp(b))


@pytest.fixture(scope="module")
def o():
    return oracle.load()


def _check(f, ref, xs, bound=1.0):
    worst = 0.0
    for x in xs:
        e = ulps(f(float(x)), ref(float(x)))
        worst = max(worst, e)
    assert worst <= bound, worst


def test_log(o):
    rng = np.random.default_rng(1)
    xs = np.exp(rng.uniform(-700, 700, 20000))
    near1 = 1.0 + rng.uniform(-0.01, 0.01, 20000)
    _check(o.oracle_math_log, math.log, np.concatenate([xs, near1, [2.0, 0.5, 1e-300, 5e-324, 1e308]]))
    assert o.oracle_math_log(1.0) == 0.0
    assert o.oracle_math_log(0.0) == -math.inf
    assert math.isnan(o.oracle_math_log(-1.0))


def test_exp(o):
    rng = np.random.default_rng(2)
    xs = np.concatenate([rng.uniform(-706, 709, 20000), rng.uniform(-0.1, 0.1, 20000)])
    _check(o.oracle_math_exp, math.exp, xs)
    assert o.oracle_math_exp(0.0) == 1.0
    assert o.oracle_math_exp(-800.0) == 0.0          # documented flush below -707
    assert o.oracle_math_exp(710.0) == math.inf


def test_expm1(o):
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.uniform(-40, 5, 20000), rng.uniform(-0.02, 0.02, 20000),
                         -np.exp(rng.uniform(-40, 0, 20000))])
    _check(o.oracle_math_expm1, math.expm1, xs)
    assert o.oracle_math_expm1(1e-20) == 1e-20
    assert o.oracle_math_expm1(-800.0) == -1.0


def test_log1p(o):
    rng = np.random.default_rng(4)
    xs = np.concatenate([np.exp(rng.uniform(-60, 60, 20000)), rng.uniform(0, 0.01, 20000)])
    _check(o.oracle_math_log1p, math.log1p, xs)
    assert o.oracle_math_log1p(0.0) == 0.0
    assert o.oracle_math_log1p(1e-300) == 1e-300


def test_tables_are_generated_from_mathematics():
    """The committed header is exactly what the generator script prints."""
    import os
    import subprocess
    import sys
    from tests.helpers import ROOT
    d = os.path.join(ROOT, "twoscalerich_gb300", "csrc")
    out = subprocess.run([sys.executable, os.path.join(d, "gen_math_tables.py")],
                         capture_output=True, text=True, check=True).stdout
    assert out == open(os.path.join(d, "tsr_math_tables.h")).read()


def test_expm1_cancelling_range(o):
    """|x| in [2^-8, ln2]: the result is formed in 128-bit fixed point from
    the 2^126-scaled table and rounded once."""
    rng = np.random.default_rng(5)
    xs = np.concatenate([rng.uniform(-0.75, 0.75, 40000), -np.exp(rng.uniform(-5.6, -0.3, 20000)),
                         [2.0 ** -8, -2.0 ** -8, math.log(2.0), -math.log(2.0), -0.35, 0.35]])
    _check(o.oracle_math_expm1, math.expm1, xs)


def test_log1p_unit_sum_is_exact_and_log_accurate(o):
    """log1p(e) for e in [0, 1] also returns 1 + e rounded to double,
    formed in fixed point: it must equal the FP64 sum exactly."""
    rng = np.random.default_rng(6)
    es = np.concatenate([rng.uniform(0, 1, 20000), np.exp(rng.uniform(-50, 0, 20000)),
                         [0.0, 1.0, 2.0 ** -8, 2.0 ** -60, 2.0 ** -61, 2.0 ** -53, 3e-17, 5e-324]])
    s1 = np.zeros(1)
    worst = 0.0
    from twoscalerich_gb300 import capi
    for e in es:
        r = o.oracle_math_log1p_unit(float(e), capi.ptr(s1))
        assert s1[0] == 1.0 + float(e), e
        worst = max(worst, ulps(r, math.log1p(float(e))))
    assert worst <= 1.0, worst


def _div_cases(rng, n):
    ex = rng.integers(-300, 300, size=(2, n))
    a = rng.uniform(1.0, 2.0, n) * np.exp2(ex[0]) * rng.choice([-1.0, 1.0], n)
    b = rng.uniform(1.0, 2.0, n) * np.exp2(ex[1]) * rng.choice([-1.0, 1.0], n)
    # divisors whose mantissa is near 1 (seed row 0), near 2, a power of two;
    # equal mantissas; quotients near the ends of the normal range
    edge_b = np.concatenate([1.0 + rng.integers(1, 2 ** 20, 2000) * 2.0 ** -52,
                             2.0 - rng.integers(1, 2 ** 20, 2000) * 2.0 ** -52,
                             np.exp2(rng.integers(-20, 20, 500).astype(float))])
    edge_a = rng.uniform(1.0, 2.0, edge_b.size) * np.exp2(rng.integers(-20, 20, edge_b.size))
    same = rng.uniform(1.0, 2.0, 1000)
    big = np.array([1.7e308, 1e308, 2.2e-308, 3e-308, 1e-300, 5e-324, 0.0, -0.0, 1.0, 3.0])
    bigd = np.array([0.9, 1.1, 1.5, 0.7, 1e10, 1.0, 2.0, 3.0, 3.0, 1.0])
    a = np.concatenate([a, edge_a, same * 2.0 ** 7, big])
    b = np.concatenate([b, edge_b, same, bigd])
    return np.ascontiguousarray(a), np.ascontiguousarray(b)


def test_integer_pipe_division_is_the_ieee_quotient(o):
    """tsr_div (Newton-Raphson reciprocal and remainder correction on the
    integer pipe) returns the correctly rounded quotient: the same bits as
    the IEEE division a / b on every case (random exponents and signs,
    divisor mantissas at both ends of [1, 2) and powers of two, equal
    mantissas, quotients at the ends of the double range, zeros).  A binary
    quotient is never exactly halfway between two doubles, so the rounding
    decision rests on the remainder alone."""
    from twoscalerich_gb300 import capi
    rng = np.random.default_rng(7)
    for _ in range(4):
        a, b = _div_cases(rng, 500_000)
        out = np.empty_like(a)
        o.oracle_math_div_many(capi.ptr(a), capi.ptr(b), capi.ptr(out), a.size)
        with np.errstate(over="ignore", under="ignore"):
            ref = a / b
        bad = np.nonzero(out.view(np.uint64) != ref.view(np.uint64))[0]
        assert bad.size == 0, (a[bad[:5]], b[bad[:5]], out[bad[:5]], ref[bad[:5]])
