"""The oracle's classical Gram-Schmidt twice (CGS2) variant of the Arnoldi
step, on the CPU: its trajectory does not depend on the thread count (every
dot is a fixed-order reduction), it stays close to the modified
Gram-Schmidt trajectory (the two differ by rounding and the step decisions
rounding moves), and an unknown variant is refused."""
import numpy as np
import pytest

import oracle
from twoscalerich_gb300 import problem as P


def _run(p, variant, threads):
    o = oracle.Oracle(p, nthreads=threads, gram_schmidt=variant)
    u, sol, st, log = P.run_to_end(o.exprem_step, p)
    return sol, st.NumSteps, st.FuncEvals, log


def _problem():
    p = P.config1(lib=oracle.MeshLib())
    p.tend = 0.004
    p.tspan = np.array([2.0, 0.002, 0.004])
    return p


def test_cgs2_bits_independent_of_threads():
    p = _problem()
    a = _run(p, 1, 1)
    b = _run(p, 1, 4)
    assert np.array_equal(a[0], b[0]) and a[1:] == b[1:]


def test_cgs2_close_to_mgs():
    p = _problem()
    c = _run(p, 1, 4)
    m = _run(p, 0, 4)
    for k in range(1, c[0].shape[0]):
        assert np.max(np.abs(c[0][k] - m[0][k])) <= 1e-6 * np.max(np.abs(m[0][k]))


def test_unknown_variant_refused():
    with pytest.raises(ValueError):
        oracle.Oracle(_problem(), gram_schmidt=2)
