"""The reference's own test scenario on the GPU, against the oracle, through
the C-ABI.

The scenario is the reference's tests/Richards_Equation (kept in
tests/golden/ref_fixture.npz by tests/golden/make_fixture.py and written
back into its file formats here): its problem_options.txt, the 10x10
quadrilateral macro mesh, the 167-node unstructured inclusion mesh and the
tabulated full Keff(h) tensor, read by this library's readers as the
reference's main() reads them (src/main.cpp:32-300) -- BC types
[1, 3, 2, 2, 2], model_type 3, h0 = -20 m, the reference's default solver
options, and the driver's boundary_flux = 1.89 (the options file has 18
values for 19 reads).  Its units are metres and seconds (Ks = 1.222e-5 m/s).

With that influx the inlet nodes saturate after about 5.5 ms; at h = 0 the
model's storage drops to the specific storage alone, the step-size
controller shrinks the step below MinStep, and the run stops with
TSR_ERR_MINSTEP.  The tests check G and Jv, the trajectory to 5 ms, and
that the GPU stops at the same step, time and state as the oracle.  BC type
4 (dh/dy = 0, src/main.cpp:178) runs on the same scenario with the south
side switched to it.

Tolerances: the same bits as the oracle (the required bounds, 1e-12 for G
and Jv and 1e-8 for trajectories, are asserted too).
"""
import numpy as np
import pytest

import oracle
from tests.helpers import write_reference_fixture
from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P

pytestmark = pytest.mark.gpu

G_RTOL = 1e-12
TRAJ_RTOL = 1e-8


def rel_err(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def fixture(tmp_path, macro_bc=(1, 3, 2, 2, 2)):
    return P.from_reference_files(write_reference_fixture(str(tmp_path)), macro_bc=macro_bc)


@pytest.mark.parametrize("macro_bc", [(1, 3, 2, 2, 2), (1, 4, 3, 3, 2)],
                         ids=["reference_bcs", "bc4_south"])
def test_fixture_g_jv_bitwise(tmp_path, macro_bc):
    p = fixture(tmp_path, macro_bc)
    assert p.ud.boundary_flux == 1.89
    ctx = P.Context(p, max_krylov=0)
    orc = oracle.Oracle(p)
    rng = np.random.default_rng(17)
    for u in (p.u0, p.u0 + rng.normal(0.0, 2.0, p.N)):
        gg, go = ctx.g(u), orc.g(u)
        assert rel_err(gg, go) <= G_RTOL
        assert np.array_equal(gg, go)
        v = rng.normal(size=p.N)
        v /= np.sqrt(orc.dot(v, v))
        eps = np.sqrt((1.0 + np.sqrt(orc.dot(u, u))) * np.finfo(float).eps)
        wg, wo = ctx.jv(u, go, v, eps), orc.jv(u, go, v, eps)
        assert rel_err(wg, wo) <= G_RTOL
        assert np.array_equal(wg, wo)


@pytest.mark.parametrize("macro_bc", [(1, 3, 2, 2, 2), (1, 4, 3, 3, 2)],
                         ids=["reference_bcs", "bc4_south"])
def test_fixture_trajectory_to_5ms(tmp_path, macro_bc):
    p = fixture(tmp_path, macro_bc)
    p.tend = 0.005
    p.tspan = np.array([2.0, 0.0025, 0.005])
    ctx = P.Context(p)
    orc = oracle.Oracle(p, nthreads=8)
    ug, sg, stg, logg = P.run_to_end(ctx.exprem_step, p)
    uo, so, sto, logo = P.run_to_end(orc.exprem_step, p)
    assert logg == logo and stg.FuncEvals == sto.FuncEvals
    assert logg[-1][1] == p.tend
    for k in range(sg.shape[0]):
        assert rel_err(sg[k], so[k]) <= TRAJ_RTOL
        wa, wb = ctx.water(sg[k]), orc.water(so[k])
        assert abs(wa - wb) <= TRAJ_RTOL * abs(wb)
    assert np.array_equal(sg, so) and np.array_equal(ug, uo)
    # the influx raised the water content
    assert orc.water(so[2]) > orc.water(so[0])


def test_fixture_saturation_stops_like_the_oracle(tmp_path):
    """Run to the scenario's own t_end = 2 s: both stop with MinStep at the
    same accepted step, with the same state and statistics."""
    p = fixture(tmp_path)
    ns = int(p.tspan[0])
    results = []
    ctx = P.Context(p)
    orc = oracle.Oracle(p, nthreads=8)
    for step in (ctx.exprem_step, orc.exprem_step):
        u = p.u0.copy()
        solns = np.zeros((ns + 1) * p.N)
        st = capi.ExpremStats()
        t, code = 0.0, None
        for _ in range(5000):
            try:
                t = step(t, u, p.tspan, solns, p.options, st)
            except capi.TsrError as e:
                code = e.code
                break
            except RuntimeError as e:          # the oracle's failure
                code = int(str(e).split()[-1])
                break
            if t >= p.tend:
                break
        results.append((code, t, st.NumSteps, st.FuncEvals, st.CurrentStep, u))
    (cg, tg, ng, fg, hg, ug), (co, to, no, fo, ho, uo) = results
    assert cg == co == 8                    # TSR_ERR_MINSTEP
    assert (tg, ng, fg, hg) == (to, no, fo, ho)
    assert np.array_equal(ug, uo)
    assert 0.004 < tg < 0.01 and np.max(ug) > -1e-3    # the inlet reached saturation
