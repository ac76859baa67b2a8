"""Learned closure on the CPU: the inverse retention curve, the oracle's
learned cells (G, water, summary), the network oracle (pinned by finite
differences and exact BF16 rounding) and the training-data pipeline."""
import ctypes as C

import mpmath
import numpy as np
import pytest

import oracle
from oracle import mlp as om
from twoscalerich_gb300 import capi, closure
from twoscalerich_gb300 import problem as P


def _theta(s, h):
    """water content of soil dict s at head h, 50 digits"""
    mpmath.mp.dps = 50
    if h >= 0:
        return s["thetas"]
    m = 1 - 1 / mpmath.mpf(s["n"])
    Se = (1 + (s["alpha"] * mpmath.mpf(-h)) ** s["n"]) ** (-m)
    return float(s["thetar"] + (s["thetas"] - s["thetar"]) * Se)


@pytest.mark.parametrize("h", [-0.01, -0.1, -0.5, -1.0, -3.0, -10.0, -50.0])
def test_inverse_retention_round_trip(orc, h):
    s = P.SOIL_B
    soil = P.make_soil(**s)
    th = _theta(s, h)
    hb = orc.oracle_vg_head(C.byref(soil), th)
    # theta(h) has slope C(h); the head is determined to ~ulp(theta)/C(h)
    assert abs(hb - h) <= 1e-9 * abs(h) + 1e-12


def test_inverse_retention_saturation(orc):
    soil = P.make_soil(**P.SOIL_B)
    assert orc.oracle_vg_head(C.byref(soil), P.SOIL_B["thetas"]) == 0.0
    assert orc.oracle_vg_head(C.byref(soil), 0.9) == 0.0
    assert np.isfinite(orc.oracle_vg_head(C.byref(soil), P.SOIL_B["thetar"]))


def _mixed(p, seed=3):
    rng = np.random.default_rng(seed)
    learned = (rng.uniform(size=p.Ne) < 0.5).astype(np.int32)
    kappa = np.column_stack([rng.uniform(0.001, 0.01, p.Ne), rng.uniform(0.1, 1.0, p.Ne)]).ravel()
    return learned, kappa


def _state(p, learned, seed=4):
    """a state in the learned layout: macro and micro heads near -2, learned
    cells' water content near that of -2 m"""
    rng = np.random.default_rng(seed)
    u = -2.0 + rng.uniform(-0.5, 0.5, p.N)
    th0 = _theta(P.SOIL_B, -2.0)
    for k in np.flatnonzero(learned):
        u[p.cell_off[k]] = th0 + rng.uniform(-0.01, 0.01)
    return u


def test_learned_cells_in_oracle_g_and_water():
    p = P.config1()
    learned, kappa = _mixed(p)
    p.set_learned(learned, kappa)
    assert p.N == p.Mn + int(learned.sum()) + int((1 - learned).sum()) * p.mn
    orc = oracle.Oracle(p, nthreads=2)
    u = _state(p, learned)
    g = orc.g(u)
    assert orc.flag == 0
    S = orc.cell_summary(u, g)
    k = np.flatnonzero(learned)
    Hc, th, rate, Q, hb = S[k].T
    assert np.array_equal(th, u[p.cell_off[k]])
    assert np.array_equal(rate, g[p.cell_off[k]])
    # relaxation towards theta_B(H_c): the oracle's own water content at H_c
    lib = oracle.load()
    soil = P.make_soil(**P.SOIL_B)
    out = np.empty(3)
    thH = np.empty(k.size)
    for i, h in enumerate(Hc):
        lib.oracle_vg(C.byref(soil), 0.0, h, out.ctypes.data_as(capi.dp))
        thH[i] = out[2]
    assert np.array_equal(rate, kappa[2 * k + 1] * (thH - th))
    assert np.array_equal(Q, kappa[2 * k] * (thH - th))
    w = orc.water(u)
    assert np.isfinite(w) and w > 0


def test_summary_of_resolved_cells():
    p = P.config1()
    orc = oracle.Oracle(p, nthreads=2)
    u = p.u0 + np.random.default_rng(1).uniform(-0.5, 0.5, p.N)
    g = orc.g(u)
    S = orc.cell_summary(u, g)
    mn = p.mn
    bnd = capi.as_array(p.micro.boundary_nodes, mn, np.int32) != 1
    cv = capi.as_array(p.micro.CV_area, mn, np.float64)
    for k in (0, 17, p.Ne - 1):
        h = u[p.cell_off[k]:p.cell_off[k] + mn][bnd]
        th = np.array([_theta(P.SOIL_B, x) for x in h])
        assert abs(S[k, 1] - (th * cv[bnd]).sum() / cv[bnd].sum()) <= 1e-14
        assert S[k, 4] < 0


def test_mlp_oracle_gradient_matches_finite_differences():
    p = om.init_params(3).astype(np.float64)
    rng = np.random.default_rng(1)
    x = rng.standard_normal((40, 8))
    y = rng.standard_normal((40, 2))
    _, g = om.loss_grad(p, x, y, bf=False)
    idx = rng.choice(np.flatnonzero(np.abs(g) > 1e-6), 25, replace=False)
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (om.loss_grad(pp, x, y, bf=False)[0] - om.loss_grad(pm, x, y, bf=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-4 * abs(g[i]) + 1e-9


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5e-3, 3.0e38],
                 dtype=np.float32)
    r = om.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0
    bits = r.view(np.uint32)
    assert np.all(bits & 0xFFFF == 0)


def test_init_params_layout_matches_oracle():
    assert closure.init_params(5).size == om.N_PARAMS
    assert np.array_equal(closure.init_params(5), om.init_params(5))


def test_samples_features_and_targets():
    """a synthetic three-cell log through closure.samples"""
    p = P.config1()
    rng = np.random.default_rng(2)
    logs = []
    for n in range(5):
        S = np.zeros((p.Ne, 5), dtype=np.float64)
        S[:, 0] = -1.0 - 0.1 * n                     # H_c falling 0.1 per step
        S[:, 4] = -2.0                               # h(theta)
        S[:, 1] = 0.2
        d = closure.theta_of(S[:, 0], P.SOIL_B) - S[:, 1]
        S[:, 3] = 0.05 * d                           # Q = 0.05 (theta_B(H_c) - theta)
        S[:, 2] = 0.5 * d
        logs.append((0.1 * n, S.astype(np.float32)))
    X, Y = closure.samples(p, logs)
    assert X.shape[1] == 8 and Y.shape[1] == 2
    assert np.allclose(Y[:, 0], np.log(0.05), atol=1e-5)
    # second target: log(Q / (s^2 A_int d theta/dt)) = log(0.1 / (s^2 A_int))
    aint = closure.interior_area(p)
    assert np.allclose(Y[:, 1].reshape(-1, p.Ne), np.log(0.1 / aint), atol=1e-5)
    # rate features: asinh(-0.1 / 0.1) = asinh(-1) once the history exists
    last = X[-p.Ne:]
    assert np.allclose(last[:, 1:4], np.arcsinh(-1.0), atol=1e-5)


def test_theta_of_matches_oracle_vg(orc):
    soil = P.make_soil(**P.SOIL_B)
    out = np.empty(3)
    for h in (-0.05, -0.7, -4.0, -30.0, 0.0, 0.3):
        orc.oracle_vg(C.byref(soil), 0.0, h, out.ctypes.data_as(capi.dp))
        assert abs(closure.theta_of(h, P.SOIL_B) - out[2]) <= 1e-14


def test_standardise_and_model_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    X = np.zeros((500, 8), dtype=np.float32)
    X[:, :6] = rng.normal(2.0, 3.0, (500, 6))
    Y = rng.normal(-8.0, 0.5, (500, 2)).astype(np.float32)
    Xs, Ys, st = closure.standardise(X, Y, margin=0.25)
    fmu, fsd, ymu, ysd, zlo, zhi = st
    assert np.allclose(Xs[:, :6].mean(0), 0.0, atol=1e-5) and np.allclose(Xs[:, :6].std(0), 1.0, atol=1e-4)
    assert np.all(Xs[:, 6:] == 0.0)
    assert np.all(Xs[:, :6].min(0) >= zlo) and np.all(Xs[:, :6].max(0) <= zhi)
    model = closure.ClosureModel(closure.init_params(4), fmu, fsd, ymu, ysd, zlo, zhi)
    path = str(tmp_path / "model.npz")
    model.save(path)
    m2 = closure.ClosureModel.load(path)
    assert np.array_equal(m2.params, model.params)
    assert np.array_equal(m2.norm(), model.norm()) and np.array_equal(m2.zrange(), model.zrange())
    assert m2.norm().size == 16 and m2.zrange().size == 12
