"""Physics and self-consistency checks of the CPU oracle.

The reference's Gfunc and exprem bodies are not in its tree, so these
checks -- not reference outputs -- are what pin the restated model and
method: hydrostatic equilibrium is stationary, the macro CVFE assembly
conserves mass exactly, the finite-difference Jv is consistent with
central differences, the OpenMP form equals the serial one, and EXPREM
agrees with an independent stiff integrator (scipy Radau)."""
import ctypes as C

import numpy as np
import pytest
from scipy.integrate import solve_ivp

import oracle
from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P


def hydrostatic_state(p, c):
    """h = c - y at every macro node and every micro node (physical y)."""
    Mn, Ne = p.Mn, p.Ne
    xy = p.array("nodes", 2 * Mn)
    u = np.empty(p.N)
    u[:Mn] = c - xy[Mn:]
    cent = p.array("centroid_elements", 2 * Ne)
    s = p._scale if p._scale is not None else np.ones(Ne)
    for k in range(Ne):
        m = p._tpl[p.cell_template[k]] if p.cell_template is not None else p.micro
        mn = m.no_nodes
        vec = capi.as_array(m.vectors, 2 * mn)
        off = int(p.cell_off[k])
        u[off:off + mn] = c - (cent[Ne + k] + s[k] * vec[mn:])
    return u


@pytest.mark.parametrize("make", [lambda: P.config2(n_macro=11, n_micro=7),
                                  lambda: P.fixture10(boundary_flux=0.0),
                                  lambda: P.config3(n_macro=9)])
def test_hydrostatic_equilibrium_is_stationary(make):
    p = make()
    c = -3.0
    p.ext.dirichlet_h = c - 1.0        # top side y = 1
    o = oracle.Oracle(p)
    scale = np.max(np.abs(o.g(p.u0)))
    g = o.g(hydrostatic_state(p, c))
    assert np.max(np.abs(g)) <= 1e-10 * scale, np.max(np.abs(g)) / scale


def test_macro_assembly_conserves_mass_exactly():
    """model_type 2 (no exchange), inflow on x in [0, 0.4] of the top, no
    flow elsewhere: sum of storage rates = boundary_flux * 0.4."""
    p = P.fixture10(boundary_flux=0.05)
    p.ud.model_type = 2
    bc = capi.as_array(p.macro.boundary_condition_edges, 4 * p.Ne, np.int32)
    assert set(np.unique(bc)) <= {0, 1, 2, 3}
    # make the south side no-flow as well
    bcm = capi.as_array(p.macro.boundary_condition_edges, 4 * p.Ne, np.int32)
    bcm[bcm == 3] = 2
    C.memmove(p.macro.boundary_condition_edges, bcm.ctypes.data, bcm.nbytes)
    p.ud.macro_mesh = p.macro
    o = oracle.Oracle(p)
    rng = np.random.default_rng(1)
    u = -5.0 + rng.normal(0, 0.5, p.N)
    g = o.g(u)
    lib = oracle.load()
    cv = p.array("CV_area", p.Mn)
    rate = 0.0
    out = np.zeros(3)
    for i in range(p.Mn):
        lib.oracle_vg(C.byref(p.soilA), 1e-6, u[i], capi.ptr(out))
        rate += p.keff.epsilonA * out[1] * cv[i] * g[i]
    assert abs(rate - 0.05 * 0.4) <= 1e-12 * 0.02


def test_jv_consistent_with_central_differences():
    p = P.config2(n_macro=11, n_micro=7)
    o = oracle.Oracle(p)
    u = p.u0
    g0 = o.g(u)
    rng = np.random.default_rng(2)
    v = rng.normal(size=p.N)
    v /= np.linalg.norm(v)
    eps = np.sqrt((1.0 + np.linalg.norm(u)) * np.finfo(float).eps)
    w = o.jv(u, g0, v, eps)
    d = 1e-5
    wc = (o.g(u + d * v) - o.g(u - d * v)) / (2 * d)
    assert np.linalg.norm(w - wc) <= 1e-5 * np.linalg.norm(wc)


def test_openmp_form_equals_serial_form():
    p = P.config2(n_macro=21, n_micro=9)
    a = oracle.Oracle(p, nthreads=1).g(p.u0)
    b = oracle.Oracle(p, nthreads=4).g(p.u0)
    assert np.array_equal(a, b)


def test_exprem_matches_independent_stiff_integrator():
    """EXPREM (tol 1e-9) against scipy's Radau IIA (rtol 1e-11) on a small
    two-scale problem to t = 0.02 d."""
    p = P.config2(n_macro=5, n_micro=5)
    p.tend = 0.02
    p.tspan = np.array([2.0, 0.01, 0.02])
    p.options = P.default_options(AbsTol=1e-9, RelTol=1e-9, MaxKrylov=40)
    o = oracle.Oracle(p)
    u_e, sol, st, _ = P.run_to_end(o.exprem_step, p)
    sol_r = solve_ivp(lambda t, y: o.g(np.ascontiguousarray(y)), (0.0, p.tend), p.u0,
                      method="Radau", rtol=1e-11, atol=1e-13, t_eval=[0.01, 0.02])
    assert sol_r.success
    for k in (1, 2):
        ref = np.ascontiguousarray(sol_r.y[:, k - 1])
        err = np.max(np.abs(sol[k] - ref)) / np.max(np.abs(ref))
        assert err <= 1e-6, (k, err)
        # total water agrees too
        assert abs(o.water(sol[k]) - o.water(ref)) <= 1e-6 * abs(o.water(ref))


def test_exprem_leaves_hydrostatic_state_in_place():
    p = P.config2(n_macro=7, n_micro=5)
    c = -3.0
    p.ext.dirichlet_h = c - 1.0
    p.u0 = hydrostatic_state(p, c)
    p.tend = 0.05
    p.tspan = np.array([1.0, 0.05])
    o = oracle.Oracle(p)
    u, sol, st, _ = P.run_to_end(o.exprem_step, p)
    assert np.max(np.abs(u - p.u0)) <= 1e-9


def test_infiltration_increases_water_and_saved_times():
    p = P.config2(n_macro=7, n_micro=5)
    p.tend = 0.1
    p.tspan = np.array([4.0, 0.025, 0.05, 0.075, 0.1])
    o = oracle.Oracle(p)
    u, sol, st, log = P.run_to_end(o.exprem_step, p)
    w = [o.water(sol[k]) for k in range(5)]
    assert all(b > a for a, b in zip(w, w[1:]))
    assert log[-1][1] == p.tend
    assert np.array_equal(sol[-1], u)   # the last saved time is t_end
    assert st.FuncEvals > st.NumSteps


@pytest.mark.parametrize("bc_south", [3, 4])
def test_free_drainage_boundary_types(bc_south):
    """BC types 3 (dh/dx = 0) and 4 (dh/dy = 0) on the south side
    (src/main.cpp:175-178), no flow elsewhere, model_type 2, head linear in
    y (h = -5 + 0.3 y) on macro and micro nodes: the macro assembly
    conserves mass, so the storage rates sum to the south outflow,
    -K22(h = -5) (1 + dh/dy) over the unit side, where type 4 zeroes dh/dy
    and type 3 keeps it (dh/dx = 0 already)."""
    p = P.fixture10(boundary_flux=0.0, macro_bc=(2, bc_south, 2, 2, 2))
    p.ud.model_type = 2
    o = oracle.Oracle(p)
    xy = p.array("nodes", 2 * p.Mn)
    u = np.full(p.N, -5.0)
    u[:p.Mn] = -5.0 + 0.3 * xy[p.Mn:]
    g = o.g(u)
    lib = oracle.load()
    cv = p.array("CV_area", p.Mn)
    rate = 0.0
    out = np.zeros(3)
    for i in range(p.Mn):
        lib.oracle_vg(C.byref(p.soilA), 1e-6, u[i], capi.ptr(out))
        rate += p.keff.epsilonA * out[1] * cv[i] * g[i]
    K = np.zeros(4)
    lib.oracle_keff(C.byref(p.keff), -5.0, capi.ptr(K))
    expect = -K[3] * (1.0 + (0.0 if bc_south == 4 else 0.3))
    assert abs(rate - expect) <= 1e-12 * abs(expect), (rate, expect)
