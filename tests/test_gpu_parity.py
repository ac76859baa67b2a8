"""GPU G / Jv / reductions against the CPU oracle, through the C-ABI.

Tolerance: the kernels evaluate the same IEEE operation sequence as the
oracle (same table-driven log/exp, same summation orders, no contraction),
so G, Jv and the fixed-order dot products are required to match bit for
bit; the required bound (1e-12 relative for G and Jv) is checked as well.
"""
import numpy as np
import pytest

import oracle
from twoscalerich_gb300 import problem as P

pytestmark = pytest.mark.gpu

G_RTOL = 1e-12


def rel_err(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def cases():
    return {
        "config1": lambda: P.config1(),
        "config1_upwind": lambda: P.config1(kface=1),
        "fixture10_quads": lambda: P.fixture10(),
        "config2_small": lambda: P.config2(n_macro=21, n_micro=9),
        "config3_batched": lambda: P.config3(n_macro=21),
    }


@pytest.mark.parametrize("name", list(cases()))
def test_g_bitwise(name):
    p = cases()[name]()
    ctx = P.Context(p, max_krylov=0)
    orc = oracle.Oracle(p)
    rng = np.random.default_rng(3)
    for u in (p.u0, p.u0 + rng.normal(0, 0.3, p.N)):
        u = np.minimum(u, -1e-3)
        gg = ctx.g(u)
        go = orc.g(u)
        assert rel_err(gg, go) <= G_RTOL
        assert np.array_equal(gg, go), "max |diff| %g" % np.max(np.abs(gg - go))


@pytest.mark.parametrize("name", list(cases()))
def test_jv_bitwise(name):
    p = cases()[name]()
    ctx = P.Context(p, max_krylov=0)
    orc = oracle.Oracle(p)
    rng = np.random.default_rng(5)
    u = p.u0.copy()
    g0 = orc.g(u)
    v = rng.normal(size=p.N)
    v /= np.sqrt(orc.dot(v, v))
    eps = np.sqrt((1.0 + np.sqrt(orc.dot(u, u))) * np.finfo(float).eps)
    wg = ctx.jv(u, g0, v, eps)
    wo = orc.jv(u, g0, v, eps)
    assert rel_err(wg, wo) <= G_RTOL
    assert np.array_equal(wg, wo)


def test_model_types():
    for mt in (1, 2, 3):
        p = P.config2(n_macro=11, n_micro=7)
        p.ud.model_type = mt
        ctx = P.Context(p, max_krylov=0)
        orc = oracle.Oracle(p)
        assert np.array_equal(ctx.g(p.u0), orc.g(p.u0))


@pytest.mark.parametrize("n", [1, 255, 8192, 8193, 100003, 1 << 20])
def test_dot_fixed_order(n):
    p = P.config2(n_macro=41, n_micro=21)      # N large enough for the biggest case
    ctx = P.Context(p, max_krylov=0)
    rng = np.random.default_rng(n)
    x = rng.normal(size=n)
    y = rng.normal(size=n)
    assert ctx.dot(x, y) == oracle.load().oracle_dot(oracle.Oracle(p)._p(x), oracle.Oracle(p)._p(y), n)


def test_water_content():
    p = P.config2(n_macro=21, n_micro=9)
    ctx = P.Context(p, max_krylov=0)
    orc = oracle.Oracle(p)
    assert ctx.water(p.u0) == orc.water(p.u0)


def test_autotuned_packings_give_identical_bits():
    """Every packing of cells into CTAs the autotuner tries gives the same G."""
    p = P.config3(n_macro=31)
    ctx = P.Context(p, max_krylov=0)
    g_default = ctx.g(p.u0)
    ms, thr, bud = ctx.autotune(p.u0, reps=2)
    assert ms > 0 and thr % 32 == 0 and 128 <= thr <= 1024 and bud >= 48 * 1024
    assert np.array_equal(ctx.g(p.u0), g_default)
    assert np.array_equal(g_default, oracle.Oracle(p, nthreads=8).g(p.u0))


@pytest.mark.parametrize("make", [lambda: P.config3(n_macro=21), lambda: P.config2(n_macro=21, n_micro=21)],
                         ids=["config3_batched", "config2_21x21_cells"])
def test_cell_plans_give_identical_bits(make):
    """Block sizes, shared-memory budgets (cells per bundle) and the place
    of the math tables (shared memory or read through L1) change the speed
    of the cell kernel, never its bits."""
    import ctypes as C
    from twoscalerich_gb300 import capi
    p = make()
    lib = capi.load()
    ctx = P.Context(p, max_krylov=0)
    ref = oracle.Oracle(p, nthreads=8).g(p.u0)
    plan = (C.c_int * 6)()
    for threads, budget, tables in ((224, 64 * 1024, 1), (224, 64 * 1024, 0), (448, 144 * 1024, 0),
                                    (160, 48 * 1024, 1), (1024, 200 * 1024, 0), (128, 0, 0), (128, 0, 1)):
        capi.check(lib.tsr_set_cell_plan(ctx.h, threads, budget, tables), "plan")
        capi.check(lib.tsr_cell_plan(ctx.h, plan), "read plan")
        assert plan[0] == threads and plan[2] == tables
        assert np.array_equal(ctx.g(p.u0), ref)
