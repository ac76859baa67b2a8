"""EXPREM on the GPU against the oracle's EXPREM, through the C-ABI.

The required bound is 1e-8 relative in h and in total water content at
every saved time.  Because G, Jv, every reduction and the host-side
decisions follow the same operation sequence, the trajectories are in fact
required to agree bit for bit (same steps, Krylov dimensions, FuncEvals).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P

pytestmark = pytest.mark.gpu

TRAJ_RTOL = 1e-8


def _compare(p, nthreads=16, max_steps=100000):
    ctx = P.Context(p)
    orc = oracle.Oracle(p, nthreads=nthreads)
    ug, sg, stg, logg = P.run_to_end(ctx.exprem_step, p, max_steps=max_steps)
    uo, so, sto, logo = P.run_to_end(orc.exprem_step, p, max_steps=max_steps)
    assert len(logg) == len(logo)
    assert stg.NumSteps == sto.NumSteps and stg.FuncEvals == sto.FuncEvals
    for k in range(sg.shape[0]):
        a, b = sg[k], so[k]
        assert np.max(np.abs(a - b)) <= TRAJ_RTOL * np.max(np.abs(b))
        wa, wb = ctx.water(a), orc.water(b)
        assert abs(wa - wb) <= TRAJ_RTOL * abs(wb)
    assert np.array_equal(sg, so)
    assert np.array_equal(ug, uo)
    assert logg == logo
    return stg, logg


def test_trajectory_config1():
    p = P.config1()
    st, log = _compare(p)
    assert log[-1][1] == p.tend


def test_trajectory_fixture10_quads():
    p = P.fixture10()
    _compare(p)


def test_trajectory_config2_small_scaled_cells():
    p = P.config2(n_macro=21, n_micro=9)
    p.tend = 0.2
    p.tspan = np.concatenate([[4.0], np.linspace(0.05, 0.2, 4)])
    _compare(p)


def test_trajectory_config3_batched_uneven_cells():
    p = P.config3(n_macro=11)
    p.tend = 0.05
    p.tspan = np.concatenate([[2.0], [0.025, 0.05]])
    _compare(p)


def test_device_resident_stepping_matches_host_stepping():
    p = P.config1()
    p.tend = 0.05
    p.tspan = np.array([1.0, 0.05])
    ctx = P.Context(p)
    lib = capi.load()
    uh, sh, sth, logh = P.run_to_end(ctx.exprem_step, p)
    ctx2 = P.Context(p)
    capi.check(lib.tsr_exprem_load(ctx2.h, capi.ptr(p.u0), 0.0), "load")
    st = capi.ExpremStats()
    solns = np.zeros(2 * p.N)
    t = C.c_double(0.0)
    while t.value < p.tend:
        capi.check(lib.tsr_exprem_advance(ctx2.h, p.tend, capi.ptr(p.tspan), capi.ptr(solns),
                                          C.byref(p.options), C.byref(st), C.byref(t)), "advance")
    u = np.empty(p.N)
    capi.check(lib.tsr_exprem_store(ctx2.h, capi.ptr(u)), "store")
    assert np.array_equal(u, uh)
    assert st.FuncEvals == sth.FuncEvals


def test_graph_replay_equals_direct_launches():
    """Arnoldi steps replayed from captured CUDA graphs give the same
    trajectory as launching their kernels one by one."""
    p = P.config2(n_macro=21, n_micro=9)
    p.tend = 0.1
    p.tspan = np.array([1.0, 0.1])
    lib = capi.load()
    runs = []
    for graphs in (0, 1):
        ctx = P.Context(p)
        capi.check(lib.tsr_set_graphs(ctx.h, graphs), "graphs")
        launches0 = lib.tsr_kernel_launches()
        runs.append(P.run_to_end(ctx.exprem_step, p) + (lib.tsr_kernel_launches() - launches0,))
    (ua, sa, sta, la, na), (ub, sb, stb, lb, nb) = runs
    assert np.array_equal(ua, ub) and np.array_equal(sa, sb) and la == lb
    assert sta.FuncEvals == stb.FuncEvals
    assert na == nb            # replays count the kernels they contain


def test_dropin_gfunc_signature_path():
    """tsr_gfunc_gpu is what the C++ Gfunc_gpu(g, u, user_data) calls."""
    p = P.config1()
    lib = capi.load()
    capi.check(lib.tsr_set_default_ext(C.byref(p.ext), 30), "ext")
    g = np.empty(p.N)
    u = p.u0.copy()
    capi.check(lib.tsr_gfunc_gpu(capi.ptr(g), capi.ptr(u), C.byref(p.ud)), "gfunc")
    assert np.array_equal(g, oracle.Oracle(p).g(u))
    lib.tsr_release_all()


def test_fused_gram_schmidt_matches_separate_kernels():
    """the single-launch Gram-Schmidt block -- spread one warp per CTA over
    the GPU (1) or in one thread-block cluster (2) -- gives the same
    trajectory, bit for bit, as the separate reduction launches (0)"""
    p = P.config1()
    p.tend = 0.05
    p.tspan = np.array([1.0, 0.05])
    out = []
    for fused in (1, 2, 0):
        ctx = P.Context(p)
        capi.check(ctx.lib.tsr_set_fused_gs(ctx.h, fused), "tsr_set_fused_gs")
        out.append(P.run_to_end(ctx.exprem_step, p))
    (ua, sa, sta, la) = out[0]
    for (ub, sb, stb, lb) in out[1:]:
        assert la == lb and np.array_equal(ua, ub) and np.array_equal(sa, sb)
        assert sta.FuncEvals == stb.FuncEvals


@pytest.mark.parametrize("make", [lambda: P.config1(), lambda: P.fixture10()], ids=["config1", "fixture10_quads"])
def test_device_calibration_equals_host(make):
    """tsr_calibrate_device (the solution writer's micro-boundary overwrite,
    one warp per cell) gives the host calibration's bits."""
    torch = pytest.importorskip("torch")
    p = make()
    lib = capi.load()
    ctx = P.Context(p, max_krylov=0)
    u = p.u0 + np.random.default_rng(4).normal(0.0, 0.5, p.N)
    host = u.copy()
    capi.check(lib.tsr_calibrate_micro_boundary(C.byref(p.ud), C.byref(p.ext), capi.ptr(host)), "host")
    d = torch.from_numpy(u.copy()).to("cuda")
    torch.cuda.synchronize()
    capi.check(lib.tsr_calibrate_device(ctx.h, C.c_void_p(d.data_ptr())), "device")
    capi.check(lib.tsr_sync(ctx.h), "sync")
    assert np.array_equal(d.cpu().numpy(), host)
    assert not np.array_equal(host, u)


def test_calibrated_dense_output_rows():
    """With calibrated output the saved rows are the oracle's rows after the
    writer's calibration, bit for bit."""
    p = P.config1()
    p.tend = 0.05
    p.tspan = np.array([2.0, 0.02, 0.05])
    lib = capi.load()
    ctx = P.Context(p)
    capi.check(lib.tsr_set_calibrated_output(ctx.h, 1), "calibrated output")
    ug, sg, stg, _ = P.run_to_end(ctx.exprem_step, p)
    uo, so, sto, _ = P.run_to_end(oracle.Oracle(p, nthreads=8).exprem_step, p)
    assert np.array_equal(ug, uo)
    for k in (1, 2):
        row = so[k].copy()
        capi.check(lib.tsr_calibrate_micro_boundary(C.byref(p.ud), C.byref(p.ext), capi.ptr(row)), "host")
        assert np.array_equal(sg[k], row)
