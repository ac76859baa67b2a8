"""Checkpoint / resume of the EXPREM state through the C-ABI: a run that is
saved, restored into a fresh context and continued follows the
uninterrupted trajectory bit for bit (one extra G evaluation per scenario
for the restored G(u))."""
import ctypes as C

import numpy as np
import pytest

from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P

pytestmark = pytest.mark.gpu


def _advance(lib, h, p, st, n):
    t = C.c_double()
    tspan = np.array([0.0])
    for _ in range(n):
        capi.check(lib.tsr_exprem_advance(h, p.tend, capi.ptr(tspan), None, C.byref(p.options),
                                          C.byref(st), C.byref(t)), "advance")
    return t.value


def test_checkpoint_resume_single(tmp_path):
    p = P.config1()
    path = str(tmp_path / "run.ckpt").encode()
    a = P.Context(p)
    lib = a.lib
    capi.check(lib.tsr_exprem_load(a.h, capi.ptr(p.u0), 0.0), "load")
    st = capi.ExpremStats()
    _advance(lib, a.h, p, st, 15)
    capi.check(lib.tsr_checkpoint_save(a.h, path, C.byref(st)), "save")
    ta = _advance(lib, a.h, p, st, 15)
    ua = a.store()
    b = P.Context(p)
    sb = capi.ExpremStats()
    capi.check(lib.tsr_checkpoint_load(b.h, path, C.byref(sb)), "restore")
    assert sb.NumSteps == 15
    tb = _advance(lib, b.h, p, sb, 15)
    ub = b.store()
    assert ta == tb and sb.NumSteps == st.NumSteps and sb.FuncEvals == st.FuncEvals + 1
    assert np.array_equal(ua, ub)
    # a checkpoint of another problem is refused
    q = P.config2(n_macro=11, n_micro=5)
    c = P.Context(q)
    sc = capi.ExpremStats()
    assert lib.tsr_checkpoint_load(c.h, path, C.byref(sc)) == 5        # TSR_ERR_ARG


def test_checkpoint_resume_ensemble(tmp_path):
    ens = P.config4(scenarios=3, n_macro=7, n_micro=5)
    path = str(tmp_path / "ens.ckpt").encode()
    a = P.Context(ens)
    a.load(ens.u0)
    st = (capi.ExpremStats * 3)()
    for _ in range(8):
        a.ensemble_advance(st)
    capi.check(a.lib.tsr_checkpoint_save(a.h, path, st), "save")
    for _ in range(8):
        ta, _, _ = a.ensemble_advance(st)
    ua = a.store()
    b = P.Context(ens)
    sb = (capi.ExpremStats * 3)()
    capi.check(b.lib.tsr_checkpoint_load(b.h, path, sb), "restore")
    for _ in range(8):
        tb, _, _ = b.ensemble_advance(sb)
    ub = b.store()
    assert np.array_equal(ta, tb) and np.array_equal(ua, ub)
    assert all(sb[s].NumSteps == st[s].NumSteps and sb[s].FuncEvals == st[s].FuncEvals + 1 for s in range(3))


def test_checkpoint_refused_by_closure_contexts(tmp_path):
    """A learned-closure context neither writes nor reads checkpoints: its
    head history, coefficients and cell layout are not in the file, so a
    resumed run would not match its state (TSR_ERR_ARG both ways)."""
    p = P.config1()
    path = str(tmp_path / "plain.ckpt").encode()
    a = P.Context(p)
    lib = a.lib
    capi.check(lib.tsr_exprem_load(a.h, capi.ptr(p.u0), 0.0), "load")
    st = capi.ExpremStats()
    _advance(lib, a.h, p, st, 3)
    capi.check(lib.tsr_checkpoint_save(a.h, path, C.byref(st)), "save")
    q = P.config1()
    q.set_learned(np.zeros(q.Ne, dtype=np.int32))      # full layout, closure enabled
    b = P.Context(q)
    assert lib.tsr_num_unknowns(b.h) == p.N             # same unknown count as the file
    capi.check(lib.tsr_exprem_load(b.h, capi.ptr(q.u0), 0.0), "load")
    sb = capi.ExpremStats()
    assert lib.tsr_checkpoint_load(b.h, path, C.byref(sb)) == 5
    assert lib.tsr_checkpoint_save(b.h, str(tmp_path / "closure.ckpt").encode(), C.byref(sb)) == 5
