"""The ensemble form on the GPU (many scenarios in one launch, each with its
own EXPREM step size and Krylov dimension) against standalone oracle runs of
each scenario, through the C-ABI.

Every reduction is segmented per scenario in the single-problem order, so
each scenario's trajectory must equal its standalone oracle trajectory bit
for bit: same states, times, step sizes, Krylov dimensions and G counts
after every step, and the same solutions at the saved times."""
import numpy as np
import pytest

import oracle
from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P

pytestmark = pytest.mark.gpu


def _ens(S=4, n_macro=7, n_micro=5):
    ens = P.config4(scenarios=S, n_macro=n_macro, n_micro=n_micro)
    ens.tspan = np.array([2.0, 0.25, 0.5])
    return ens


def _standalone(ens, s):
    """Oracle trajectory of scenario s alone: per step (u, t, NumSteps,
    FuncEvals, CurrentStep, CurrentKryDim), and the tspan rows."""
    p = P.scenario_problem(ens, s)
    p.tspan = ens.tspan
    o = oracle.Oracle(p, nthreads=4)
    u = p.u0.copy()
    ns = int(p.tspan[0])
    solns = np.zeros((ns + 1) * p.N)
    st = capi.ExpremStats()
    t = 0.0
    steps = []
    while t < p.tend:
        t = o.exprem_step(t, u, p.tspan, solns, p.options, st)
        steps.append((u.copy(), t, st.NumSteps, st.FuncEvals, st.CurrentStep, st.CurrentKryDim))
    return steps, solns.reshape(ns + 1, p.N)


def test_ensemble_g_jv_water_bitwise():
    ens = _ens()
    ctx = P.Context(ens)
    orc = oracle.Oracle(ens, nthreads=4)
    rng = np.random.default_rng(11)
    u = ens.u0 + rng.uniform(-0.5, 0.5, ens.N)
    v = rng.standard_normal(ens.N)
    g = ctx.g(u)
    go = orc.g(u)
    assert np.array_equal(g, go)
    assert np.array_equal(ctx.jv(u, g, v, 3e-8), orc.jv(u, go, v, 3e-8))
    assert np.array_equal(ctx.ensemble_water(u), orc.water_scenarios(u))
    assert ctx.water(u) == orc.water(u)


@pytest.mark.parametrize("graphs", [True, False])
def test_ensemble_trajectories_equal_standalone_runs(graphs):
    ens = _ens()
    S, ns = ens.S, int(ens.tspan[0])
    ref = [_standalone(ens, s) for s in range(S)]
    ctx = P.Context(ens)
    capi.check(ctx.lib.tsr_set_graphs(ctx.h, int(graphs)), "tsr_set_graphs")
    ctx.load(ens.u0)
    stats = (capi.ExpremStats * S)()
    n_s = ens.N // S
    rows = [np.zeros((ns + 1) * n_s) for _ in range(S)]
    rounds = 0
    while True:
        t, status, nrun = ctx.ensemble_advance(stats, ens.tspan, rows)
        assert (status == 0).all()
        u = ctx.store()
        for s in range(S):
            steps = ref[s][0]
            k = min(rounds, len(steps) - 1)
            us, ts, nsteps, fevals, cstep, kdim = steps[k]
            assert t[s] == ts, (s, rounds)
            assert stats[s].NumSteps == nsteps and stats[s].FuncEvals == fevals
            assert stats[s].CurrentStep == cstep and stats[s].CurrentKryDim == kdim
            assert np.array_equal(ens.scenario(u, s), us), (s, rounds)
        rounds += 1
        if nrun == 0:
            break
    assert rounds == max(len(r[0]) for r in ref)
    # scenarios finish at different rounds (independent step sizes)
    assert len({len(r[0]) for r in ref}) > 1
    for s in range(S):
        assert np.array_equal(rows[s].reshape(ns + 1, n_s)[1:], ref[s][1][1:])


def test_ensemble_status_per_scenario():
    ens = _ens(S=3)
    ens.options.MaxNumSteps = 4
    ctx = P.Context(ens)
    ctx.load(ens.u0)
    stats = (capi.ExpremStats * ens.S)()
    for _ in range(4):
        t, status, nrun = ctx.ensemble_advance(stats)
        assert (status == 0).all() and nrun == ens.S
    t, status, nrun = ctx.ensemble_advance(stats)
    assert (status == 9).all() and nrun == 0          # TSR_ERR_MAXSTEPS
    assert all(stats[s].NumSteps == 4 for s in range(ens.S))


def test_single_problem_advance_refused_on_ensemble():
    ens = _ens(S=2)
    ctx = P.Context(ens)
    ctx.load(ens.u0)
    st = capi.ExpremStats()
    import ctypes as C
    rc = ctx.lib.tsr_exprem_advance(ctx.h, ens.tend, capi.ptr(ens.tspan), None, C.byref(ens.options),
                                    C.byref(st), None)
    assert rc == 5                                   # TSR_ERR_ARG
