"""Parity at the benchmarked sizes, through the C-ABI (marked slow).

The benchmark workloads take code paths the small parity cases do not:
autotuned bundles of cells per CTA at large shared-memory budgets, the
Gram-Schmidt block as a cooperative launch over the whole GPU (small cases
fit one thread-block cluster), 64-bit unknown offsets past 2^31 bytes,
dozens of scenarios in one launch.  These tests run the benchmarked
configurations themselves and require the same bits as the oracle:

  * 201 x 201 macro x 21 x 21 micro (N = 35,320,401): G, Jv, and the first
    three accepted EXPREM steps (Krylov dimension up to 40), device-resident
    stepping as the benchmark times it;
  * 151 x 151, uneven micro meshes (N ~ 12.8 M): G and Jv;
  * 64 scenarios of 51 x 51 x 15 x 15 (N = 72,166,464): G, Jv, and two
    lockstep rounds, four scenarios checked against standalone oracle runs.

The required bounds (1e-12 for G and Jv, 1e-8 for trajectories and water)
are asserted as well as equality.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

G_RTOL = 1e-12
TRAJ_RTOL = 1e-8
THREADS = os.cpu_count() or 1


def rel_err(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _g_jv(p, ctx, orc):
    g_gpu = ctx.g(p.u0)
    g_cpu = orc.g(p.u0)
    assert rel_err(g_gpu, g_cpu) <= G_RTOL
    assert np.array_equal(g_gpu, g_cpu), "max |diff| %g" % np.max(np.abs(g_gpu - g_cpu))
    del g_gpu
    v = np.random.default_rng(5).normal(size=p.N)
    v /= np.sqrt(orc.dot(v, v))
    eps = np.sqrt((1.0 + np.sqrt(orc.dot(p.u0, p.u0))) * np.finfo(float).eps)
    w_gpu = ctx.jv(p.u0, g_cpu, v, eps)
    w_cpu = orc.jv(p.u0, g_cpu, v, eps)
    assert rel_err(w_gpu, w_cpu) <= G_RTOL
    assert np.array_equal(w_gpu, w_cpu)


def test_config2_full_size_g_jv_and_three_steps():
    p = P.config2()                                  # 201 x 201 x 21 x 21
    assert p.N == 35_320_401
    ctx = P.Context(p)
    ctx.autotune(p.u0, reps=1)                       # the benchmark's packing
    orc = oracle.Oracle(p, nthreads=THREADS)
    _g_jv(p, ctx, orc)
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
        assert (st_g.NumSteps, st_g.FuncEvals, st_g.CurrentKryDim, st_g.CurrentStep) == \
            (st_o.NumSteps, st_o.FuncEvals, st_o.CurrentKryDim, st_o.CurrentStep)
    u_g = np.empty(p.N)
    capi.check(lib.tsr_exprem_store(ctx.h, capi.ptr(u_g)), "store")
    assert rel_err(u_g, u_o) <= TRAJ_RTOL
    assert np.array_equal(u_g, u_o)
    assert st_g.CurrentKryDim >= 1 and st_g.NumSteps == 3


def test_config3_full_size_g_jv():
    p = P.config3()                                  # 151 x 151, uneven cells
    ctx = P.Context(p, max_krylov=0)
    ctx.autotune(p.u0, reps=1)
    orc = oracle.Oracle(p, nthreads=THREADS)
    _g_jv(p, ctx, orc)


def test_config4_full_size_g_and_two_rounds():
    ens = P.config4()                                # 64 x 51 x 51 x 15 x 15
    assert ens.S == 64 and ens.N == 72_166_464
    ctx = P.Context(ens)
    ctx.autotune(ens.u0, reps=1)
    orc = oracle.Oracle(ens, nthreads=THREADS)
    _g_jv(ens, ctx, orc)
    del orc
    stats = (capi.ExpremStats * ens.S)()
    ctx.load(ens.u0)
    for _ in range(2):
        t, status, nrun = ctx.ensemble_advance(stats)
        assert np.all(status == 0)
    u = ctx.store()
    for s in (0, 21, 42, 63):
        p = P.scenario_problem(ens, s)
        o = oracle.Oracle(p, nthreads=THREADS)
        us = p.u0.copy()
        st = capi.ExpremStats()
        ts = 0.0
        sol = np.zeros(p.N)
        for _ in range(2):
            ts = o.exprem_step(ts, us, np.array([0.0]), sol, p.options, st)
        assert ts == t[s]
        assert (st.NumSteps, st.FuncEvals, st.CurrentKryDim, st.CurrentStep) == \
            (stats[s].NumSteps, stats[s].FuncEvals, stats[s].CurrentKryDim, stats[s].CurrentStep)
        got = ens.scenario(u, s)
        assert rel_err(got, us) <= TRAJ_RTOL
        assert np.array_equal(got, us)
        o.close()
