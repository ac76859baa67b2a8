"""The integration notes' change to the reference's own driver, applied to a
copy of it and built with the reference's own sources (runs where the
reference tree is present; the tree itself is never modified).

The copy of src/main.cpp gains the GB300 branch exactly as the notes show
(parallel = 2 selects Gfunc_gpu and exprem_gpu) and is compiled with the
reference's mesh preprocessing, Keff reader, options, phipade and solution
writer, with libtsr_gb300.so, and with the oracle behind the reference's
missing Gfunc_serial / Gfunc_parallel / exprem (tests/dropin/
oracle_adapters.cpp).  Run on the reference's own test scenario (its
problem_options.txt with the end time shortened to 5 ms, before the inlet
saturates; its 15 values keep the driver's boundary_flux = 1.89):

  * parallel = 1: the reference's loop on the CPU.  Its solution.txt (the
    reference's own writer, after its own micro-boundary calibration) must
    hold the trajectory the oracle computes from the same reference-built
    geometry through this repository's Python driver loop: the evolved
    entries to the last bit, the calibrated micro-boundary entries to 1e-10
    (the two interpolant formulas differ in rounding);
  * parallel = 2 in a process without a GPU: exprem_gpu reports the failure
    and the reference's loop stops (the GPU run itself is
    tests/test_gpu_dropin.py, which needs no reference tree).
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from tests.helpers import FIXTURE, ROOT, reference_root
from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P

GXX = shutil.which("g++")
pytestmark = pytest.mark.skipif(reference_root() is None or GXX is None or oracle.load_ref() is None,
                                reason="reference tree, g++ or oracle/_ref not present")


def _patch_main(src):
    """The change of INTEGRATION.md, applied to the text of src/main.cpp."""
    s = src
    s = s.replace('#include "main.h"',
                  '#include "main.h"\n#define TSR_TYPES_FROM_REFERENCE\n#include "tsr_dropin.hpp"', 1)
    sel = "    int (*Gfunc_type)(double* g, double* u, user_data_struct user_data);\n"
    assert s.count(sel) == 1
    s = s.replace(sel, sel + "    bool gpu = false;\n", 1)
    old_else = ("    else if (parallel == 1)\n    {\n        Gfunc_type = Gfunc_parallel;\n    }\n")
    assert s.count(old_else) == 1
    s = s.replace(old_else, old_else + "    else if (parallel == 2) { Gfunc_type = Gfunc_gpu; gpu = true; }   // GB300\n", 1)
    call = ("        flag = exprem(Gfunc_type, N, t, tend, tspan, tspan_solns, u0, \\\n"
            "                user_data, exprem_options, exprem_stats);\n")
    assert s.count(call) == 1
    s = s.replace(call, "        flag = gpu ? exprem_gpu(Gfunc_type, N, t, tend, tspan, tspan_solns, u0,\n"
                        "                                user_data, exprem_options, exprem_stats)\n"
                        "                   : exprem(Gfunc_type, N, t, tend, tspan, tspan_solns, u0,\n"
                        "                            user_data, exprem_options, exprem_stats);\n", 1)
    return s


def _openblas():
    import scipy
    d = os.path.abspath(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs"))
    libs = [f for f in os.listdir(d) if f.startswith("libscipy_openblas") and f.endswith(".so")]
    return d, os.path.join(d, libs[0])


def _build(tmp):
    ref = reference_root()
    src, inc = os.path.join(tmp, "src"), os.path.join(tmp, "include")
    shutil.copytree(os.path.join(ref, "src"), src)
    shutil.copytree(os.path.join(ref, "include"), inc)
    main = os.path.join(src, "main.cpp")
    text = open(main).read()
    open(main, "w").write(_patch_main(text))
    bdir, blas = _openblas()
    exe = os.path.join(tmp, "run")
    cmd = [GXX, "-O2", "-fopenmp", "-w", "-I", inc, "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-DTSR_ADAPTERS_WITH_REFERENCE_HEADERS"]
    cmd += sorted(os.path.join(src, f) for f in os.listdir(src) if f.endswith(".cpp"))
    cmd += [os.path.join(ROOT, "tests", "dropin", "oracle_adapters.cpp"), "-o", exe,
            os.path.join(ROOT, "twoscalerich_gb300", "libtsr_gb300.so"),
            os.path.join(ROOT, "oracle", "libtsr_oracle.so"), blas,
            "-Wl,-rpath," + os.path.join(ROOT, "twoscalerich_gb300"),
            "-Wl,-rpath," + os.path.join(ROOT, "oracle"), "-Wl,-rpath," + bdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _scenario(tmp, tend, times):
    run = os.path.join(tmp, "run_dir")
    shutil.copytree(os.path.join(reference_root(), "tests", "Richards_Equation"), run)
    opt = os.path.join(run, "problem_options.txt")
    tok = open(opt).read().split()
    # names, h0, tend, no_solns, times..., soil A, soil B (15 values, as the original)
    vals = tok[3:]
    new = tok[:3] + [vals[0], repr(tend), str(len(times))] + [repr(t) for t in times] + vals[3 + 2:]
    os.chmod(opt, 0o644)
    open(opt, "w").write("\n".join(new) + "\n")
    return run


def _oracle_rows(tend, times):
    """The oracle's trajectory on the reference-built geometry through this
    repository's driver loop, rows calibrated by this library."""
    g = np.load(FIXTURE)
    keep = []
    arr = lambda a: keep.append(np.ascontiguousarray(a)) or capi.ptr(keep[-1])
    M, m = capi.MacroMesh(), capi.MicroMesh()
    M.no_verts, M.no_nodes, M.no_elements = (int(x) for x in g["refgeom/macro/counts"])
    for f in ("elements", "boundary_condition_edges"):
        setattr(M, f, C.cast(arr(g["refgeom/macro/%s" % f].astype(np.int32)), capi.ip))
    for f in ("nodes", "shape_funcs", "normals", "boundary_edge_midpts", "boundary_edge_normals",
              "boundary_edge_lens", "CV_area", "SCV_area", "midx", "midy", "centroid_elements"):
        setattr(M, f, arr(g["refgeom/macro/%s" % f]))
    m.no_verts, m.no_nodes, m.no_elements = (int(x) for x in g["refgeom/micro/counts"])
    for f in ("elements", "boundary_nodes", "boundary_edges"):
        setattr(m, f, C.cast(arr(g["refgeom/micro/%s" % f].astype(np.int32)), capi.ip))
    for f in ("nodes", "shape_funcs", "normals", "boundary_edge_midpts", "boundary_edge_normals",
              "boundary_edge_lens", "centroid_elements", "CV_area", "midx", "midy", "vectors"):
        setattr(m, f, arr(g["refgeom/micro/%s" % f]))
    m.cell_area = g["refgeom/micro/cell_area"][0]
    K = capi.Keff()
    hdr = g["keff/header"]
    K.epsilonA, K.no_hvalues, K.logr, K.logh_first = hdr[0], int(hdr[1]), hdr[2], hdr[3]
    K.logh_values, K.Keff_values = arr(g["keff/logh"]), arr(g["keff/values"])
    ud = capi.UserData()
    ud.macro_mesh, ud.micro_mesh, ud.effective_conductivity = M, m, K
    ud.soilA = P.make_soil(*g["options/soilA"])
    ud.soilB = P.make_soil(*g["options/soilB"])
    ud.boundary_flux = g["options/boundary_flux"][0]
    ud.model_type, ud.NUM_THREADS = 3, 2
    N = M.no_nodes + M.no_elements * m.no_nodes
    ud.N = N
    lib = oracle.load()
    h = lib.oracle_create(C.byref(ud), None)
    opts = P.default_options()
    u = np.full(N, g["options/h0"][0])
    tspan = np.array([float(len(times))] + list(times))
    solns = np.zeros((len(times) + 1) * N)
    solns[:N] = u
    st = capi.ExpremStats()
    t = C.c_double(0.0)
    while t.value < tend:
        assert lib.oracle_exprem_step(h, C.byref(t), tend, capi.ptr(tspan), capi.ptr(solns), capi.ptr(u),
                                      C.byref(opts), C.byref(st), 2) == 0
    rows = solns.reshape(len(times) + 1, N).copy()
    for r in rows:
        capi.check(capi.load().tsr_calibrate_micro_boundary(C.byref(ud), None, capi.ptr(r)), "calibrate")
    raw = solns.reshape(len(times) + 1, N)
    lib.oracle_destroy(h)
    return rows, raw, st, keep


def test_patched_reference_main_runs_the_oracle_and_fails_cleanly_without_gpu(tmp_path):
    tmp = str(tmp_path)
    exe = _build(tmp)
    tend, times = 0.005, [0.0025, 0.005]
    run = _scenario(tmp, tend, times)
    env = dict(os.environ, parallel="1", OMP_NUM_THREADS="2")
    r = subprocess.run([exe, "problem_options.txt"], cwd=run, capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "Simulation completed successfully" in r.stdout
    tok = open(os.path.join(run, "solution.txt")).read().split()
    assert int(tok[0]) == len(times) + 1
    rows, raw, st, _ = _oracle_rows(tend, times)
    N = rows.shape[1]
    vals = np.array(tok[1:], dtype=float).reshape(len(times) + 1, N + 1)
    assert list(vals[:, 0]) == [0.0] + times
    written = vals[:, 1:]
    calibrated = written != raw
    assert np.array_equal(written[~calibrated], raw[~calibrated])
    assert np.max(np.abs(written - rows)) <= 1e-10 * np.max(np.abs(rows))
    steps = open(os.path.join(run, "statistics.txt")).read().splitlines()
    assert len(steps) == st.NumSteps
    assert "FuncEvals: %d" % st.FuncEvals in r.stdout
    # the GPU branch in a process without a GPU: exprem_gpu reports and the loop stops
    env["parallel"] = "2"
    r2 = subprocess.run([exe, "problem_options.txt"], cwd=run, capture_output=True, text=True, env=env,
                        timeout=600)
    from tests.conftest import gpu_available
    if not gpu_available():
        assert "exprem_gpu:" in r2.stderr
        assert "Simulation completed successfully" not in r2.stdout
