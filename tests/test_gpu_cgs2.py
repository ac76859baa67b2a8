"""Classical Gram-Schmidt twice (CGS2) in the Arnoldi step, on the GPU
against the oracle's CGS2, through the C-ABI.

The variant forms H(i, j) = c_i + d_i from two classical passes, each dot a
fixed-order reduction; the oracle restates it operation by operation, so
trajectories must agree bit for bit (same steps, Krylov dimensions,
FuncEvals, states).  Covered: the cluster kernel (problems of at most 16
chunks), the cooperative kernel over many chunks, segmented scenarios, and
the full benchmarked size with several chunks per CTA.  Against modified
Gram-Schmidt (the default) the trajectories differ by rounding and by the
step decisions rounding moves; that difference is bounded here as well.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P

pytestmark = pytest.mark.gpu

TRAJ_RTOL = 1e-8
THREADS = os.cpu_count() or 1


def _compare(p, max_steps=100000):
    ctx = P.Context(p, gram_schmidt=1)
    orc = oracle.Oracle(p, nthreads=THREADS, gram_schmidt=1)
    ug, sg, stg, logg = P.run_to_end(ctx.exprem_step, p, max_steps=max_steps)
    uo, so, sto, logo = P.run_to_end(orc.exprem_step, p, max_steps=max_steps)
    assert stg.NumSteps == sto.NumSteps and stg.FuncEvals == sto.FuncEvals
    for k in range(sg.shape[0]):
        assert np.max(np.abs(sg[k] - so[k])) <= TRAJ_RTOL * np.max(np.abs(so[k]))
    assert np.array_equal(sg, so)
    assert np.array_equal(ug, uo)
    assert logg == logo
    return sg, stg


def test_cgs2_trajectory_config1_cluster_kernel():
    p = P.config1()                     # 97,241 unknowns: 12 chunks, one cluster
    sg, st = _compare(p)
    # the default (modified Gram-Schmidt) run reaches the same states to
    # within the step tolerance's reach
    ctx = P.Context(p)
    um, sm, stm, logm = P.run_to_end(ctx.exprem_step, p)
    for k in range(sm.shape[0]):
        assert np.max(np.abs(sg[k] - sm[k])) <= 1e-6 * np.max(np.abs(sm[k]))
    assert abs(st.NumSteps - stm.NumSteps) <= 0.05 * stm.NumSteps


def test_cgs2_trajectory_cooperative_kernel():
    p = P.config2(n_macro=41, n_micro=9)     # ~260 k unknowns: 32 chunks
    assert p.N > 16 * 8192
    p.tend = 0.05
    p.tspan = np.array([2.0, 0.025, 0.05])
    _compare(p)


def test_cgs2_ensemble_equals_standalone_runs():
    ens = P.config4(scenarios=3, n_macro=21, n_micro=9)     # 8 chunks per scenario
    ens.tend = 0.02
    S = ens.S
    ctx = P.Context(ens, gram_schmidt=1)
    ctx.load(ens.u0)
    stats = (capi.ExpremStats * S)()
    while True:
        t, status, nrun = ctx.ensemble_advance(stats)
        assert (status == 0).all()
        if nrun == 0:
            break
    u = ctx.store()
    for s in range(S):
        p = P.scenario_problem(ens, s)
        o = oracle.Oracle(p, nthreads=THREADS, gram_schmidt=1)
        us = p.u0.copy()
        st = capi.ExpremStats()
        ts = 0.0
        sol = np.zeros(p.N)
        while ts < p.tend:
            ts = o.exprem_step(ts, us, np.array([0.0]), sol, p.options, st)
        assert ts == t[s]
        assert (st.NumSteps, st.FuncEvals, st.CurrentKryDim) == \
            (stats[s].NumSteps, stats[s].FuncEvals, stats[s].CurrentKryDim)
        assert np.array_equal(ens.scenario(u, s), us)
        o.close()


def test_cgs2_refuses_krylov_dimensions_above_63():
    p = P.config1()
    ctx = P.Context(p, max_krylov=64)
    assert ctx.lib.tsr_set_gram_schmidt(ctx.h, 1) == 5           # TSR_ERR_ARG
    assert ctx.lib.tsr_set_gram_schmidt(ctx.h, 2) == 5
    assert ctx.lib.tsr_set_gram_schmidt(ctx.h, 0) == 0


@pytest.mark.slow
def test_cgs2_full_size_three_steps():
    p = P.config2()                                  # 201 x 201 x 21 x 21, 4,312 chunks
    ctx = P.Context(p, gram_schmidt=1)
    ctx.autotune(p.u0, reps=1)
    orc = oracle.Oracle(p, nthreads=THREADS, gram_schmidt=1)
    lib = capi.load()
    tspan = np.array([0.0])
    solns = np.zeros(1)
    capi.check(lib.tsr_exprem_load(ctx.h, capi.ptr(p.u0), 0.0), "load")
    st_g, st_o = capi.ExpremStats(), capi.ExpremStats()
    t = C.c_double(0.0)
    u_o = p.u0.copy()
    t_o = 0.0
    for _ in range(3):
        capi.check(lib.tsr_exprem_advance(ctx.h, p.tend, capi.ptr(tspan), capi.ptr(solns),
                                          C.byref(p.options), C.byref(st_g), C.byref(t)), "advance")
        t_o = orc.exprem_step(t_o, u_o, tspan, solns, p.options, st_o)
        assert t.value == t_o
        assert (st_g.NumSteps, st_g.FuncEvals, st_g.CurrentKryDim) == \
            (st_o.NumSteps, st_o.FuncEvals, st_o.CurrentKryDim)
    u_g = np.empty(p.N)
    capi.check(lib.tsr_exprem_store(ctx.h, capi.ptr(u_g)), "store")
    assert np.array_equal(u_g, u_o)
