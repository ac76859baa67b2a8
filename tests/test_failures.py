"""Failure handling without any GPU fault: the failures are made on the
host (a non-finite state, a tolerance no step can meet, a step budget of
zero) and must come back as status codes, never as exit() or a trap.
Reference conventions: Gfunc returns a non-zero flag, exprem returns -1
(src/main.cpp:319-322), phipade exits on a singular denominator
(src/phipade.cpp:160-166)."""
import numpy as np
import pytest

import oracle
from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P


def _problem():
    p = P.config2(n_macro=7, n_micro=5)
    p.tend = 0.05
    p.tspan = np.array([1.0, 0.05])
    return p


def test_oracle_flags_non_finite_state():
    p = _problem()
    o = oracle.Oracle(p)
    u = p.u0.copy()
    u[p.Mn + 7] = np.nan
    o.g(u)
    assert o.flag != 0


def test_oracle_exprem_error_codes():
    p = _problem()
    o = oracle.Oracle(p)
    u = p.u0.copy()
    u[p.Mn + 7] = np.nan
    with pytest.raises(RuntimeError, match="10"):          # G(u) failed
        P.run_to_end(o.exprem_step, p, u0=u)
    p.options.AbsTol = p.options.RelTol = 1e-300           # no step can pass
    p.options.MinStep = 1e-4
    with pytest.raises(RuntimeError, match="8"):           # below MinStep
        P.run_to_end(o.exprem_step, p)
    p = _problem()
    p.options.MaxNumSteps = 0
    with pytest.raises(RuntimeError, match="9"):
        P.run_to_end(o.exprem_step, p)


@pytest.mark.gpu
def test_gpu_status_codes():
    p = _problem()
    ctx = P.Context(p)
    u = p.u0.copy()
    u[p.Mn + 7] = np.nan
    with pytest.raises(capi.TsrError) as e:
        ctx.g(u)
    assert e.value.code == 2                                # TSR_ERR_NAN
    with pytest.raises(capi.TsrError) as e:
        P.run_to_end(ctx.exprem_step, p, u0=u)
    assert e.value.code == 10                               # TSR_ERR_GFUNC
    # the context stays usable after the failures
    assert np.array_equal(ctx.g(p.u0), oracle.Oracle(p).g(p.u0))
    p.options.AbsTol = p.options.RelTol = 1e-300
    p.options.MinStep = 1e-4
    ctx2 = P.Context(p)
    with pytest.raises(capi.TsrError) as e:
        P.run_to_end(ctx2.exprem_step, p)
    assert e.value.code == 8                                # TSR_ERR_MINSTEP
    p = _problem()
    p.options.MaxNumSteps = 0
    ctx3 = P.Context(p)
    with pytest.raises(capi.TsrError) as e:
        P.run_to_end(ctx3.exprem_step, p)
    assert e.value.code == 9


@pytest.mark.gpu
def test_bounded_waits_expire_without_fault():
    """a wait that can never complete (a CTA that never reaches the grid
    barrier; an MMA barrier nothing arrives on) runs out, raises its flag
    and returns TSR_ERR_TIMEOUT; the device and a context stay usable"""
    lib = capi.load()
    assert lib.tsr_wait_probe(0) == 4                       # TSR_ERR_TIMEOUT
    assert lib.tsr_wait_probe(1) == 4
    p = _problem()
    ctx = P.Context(p)
    assert np.array_equal(ctx.g(p.u0), oracle.Oracle(p).g(p.u0))
