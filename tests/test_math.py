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
