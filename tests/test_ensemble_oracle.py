"""Ensemble form on the oracle (CPU): S independent scenarios laid out
scenario by scenario must each give exactly the standalone problem's G, Jv
and water content, so that the GPU ensemble can be checked scenario by
scenario against standalone oracle runs."""
import numpy as np

import oracle
from twoscalerich_gb300 import problem as P


def _ens():
    return P.config4(scenarios=3, n_macro=6, n_micro=5)


def test_layout_is_scenario_major():
    ens = _ens()
    n_s = ens.N // ens.S
    assert list(ens.scen_start) == [s * n_s for s in range(ens.S + 1)]
    for s in range(ens.S):
        p = P.scenario_problem(ens, s)
        assert p.N == n_s
        assert np.array_equal(p.u0, ens.scenario(ens.u0, s))


def test_union_g_jv_water_equal_standalone():
    ens = _ens()
    oe = oracle.Oracle(ens, nthreads=2)
    rng = np.random.default_rng(5)
    u = ens.u0 + rng.uniform(-0.3, 0.3, ens.N)
    v = rng.standard_normal(ens.N)
    ge = oe.g(u)
    assert oe.flag == 0
    je = oe.jv(u, ge, v, 1e-7)
    we = oe.water_scenarios(u)
    assert np.isfinite(ge).all()
    for s in range(ens.S):
        p = P.scenario_problem(ens, s)
        o = oracle.Oracle(p, nthreads=2)
        us = np.ascontiguousarray(ens.scenario(u, s))
        gs = o.g(us)
        assert np.array_equal(gs, ens.scenario(ge, s))
        js = o.jv(us, gs, np.ascontiguousarray(ens.scenario(v, s)), 1e-7)
        assert np.array_equal(js, ens.scenario(je, s))
        assert we[s] == o.water(us)
    # the total is the fixed-order sum of all scenarios' terms
    assert abs(oe.water(u) - we.sum()) <= 1e-13 * abs(we.sum())


def test_scenario_parameters_follow_the_stated_distributions():
    ens = P.config4()
    pr = ens.scenario_params
    assert ens.S == 64 and ens.N == 64 * (51 * 51 + 2 * 50 * 50 * 15 * 15)
    assert ((pr["alpha_A"] >= 1.5) & (pr["alpha_A"] <= 4.0)).all()
    assert ((pr["n_A"] >= 1.8) & (pr["n_A"] <= 2.6)).all()
    assert ((pr["h0"] >= -10.0) & (pr["h0"] <= -1.0)).all()
    assert abs(np.median(np.log(pr["Ks_A"])) - np.log(0.054)) < 0.3
    assert abs(np.median(np.log(pr["Ks_B"])) - np.log(0.001)) < 0.3
