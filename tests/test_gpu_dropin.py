"""The reference-signature drop-ins, Gfunc_gpu and exprem_gpu (C++,
include/tsr_dropin.hpp), called from a driver with the reference's own
loop (tests/dropin/dropin_driver.cpp: the right-hand side chosen by the
environment variable `parallel` as src/main.cpp:198-213 chooses it, plus the
GPU branch the integration notes add; one exprem call per step as
src/main.cpp:313-341; the solution rows calibrated as save_solution does).

parallel = 0 and 1 run the oracle behind the reference's Gfunc_serial /
Gfunc_parallel / exprem signatures (tests/dropin/oracle_adapters.cpp);
parallel = 2 runs the GB300 path through exprem_gpu, whose device context is
created implicitly from user_data (keyed by its macro element array).

The problem is the reference's own test scenario with the geometry the
reference's own mesh preprocessing produced (tests/golden/ref_fixture.npz:
its triangle SCV areas are one sixth of a triangle, the reference's quirk),
h0 = -20 m, boundary_flux = 1.89, the reference's default solver options,
run to 5 ms (before the inlet saturates).  Required: the GPU run's G at the
initial state, every step line and the saved solution rows are the same
bits as the oracle's."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests.helpers import FIXTURE, ROOT, write_reference_fixture

pytestmark = pytest.mark.gpu

MACRO = ["elements", "nodes", "shape_funcs", "normals", "boundary_edge_midpts",
         "boundary_edge_normals", "boundary_edge_lens", "boundary_condition_edges", "CV_area",
         "SCV_area", "midx", "midy", "centroid_elements"]
MICRO = ["elements", "boundary_nodes", "nodes", "shape_funcs", "normals", "boundary_edges",
         "boundary_edge_midpts", "boundary_edge_normals", "boundary_edge_lens",
         "centroid_elements", "CV_area", "midx", "midy", "vectors"]


def _write_problem(d, tend, tspan):
    g = np.load(FIXTURE)
    write_reference_fixture(d)                      # Keff.txt (and the text files)
    for f in MACRO:
        g["refgeom/macro/%s" % f].tofile(os.path.join(d, "macro_%s.bin" % f))
    for f in MICRO:
        g["refgeom/micro/%s" % f].tofile(os.path.join(d, "micro_%s.bin" % f))
    nv, Mn, Ne = (int(x) for x in g["refgeom/macro/counts"])
    _, mn, mNe = (int(x) for x in g["refgeom/micro/counts"])
    with open(os.path.join(d, "problem.txt"), "w") as f:
        f.write("%d %d %d %d %d %.17g %.17g %.17g %.17g %d\n" % (
            nv, Mn, Ne, mn, mNe, g["refgeom/micro/cell_area"][0], g["options/h0"][0], tend,
            g["options/boundary_flux"][0], len(tspan)))
        f.write(" ".join("%.17g" % t for t in tspan) + "\n")
        f.write(" ".join("%.17g" % v for v in g["options/soilA"]) + "\n")
        f.write(" ".join("%.17g" % v for v in g["options/soilB"]) + "\n")
    return Mn + Ne * mn


def _build_driver(d):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = os.path.join(d, "driver")
    cmd = [gxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "dropin", "dropin_driver.cpp"),
           os.path.join(ROOT, "tests", "dropin", "oracle_adapters.cpp"), "-o", exe,
           os.path.join(ROOT, "twoscalerich_gb300", "libtsr_gb300.so"),
           os.path.join(ROOT, "oracle", "libtsr_oracle.so"),
           "-Wl,-rpath," + os.path.join(ROOT, "twoscalerich_gb300"),
           "-Wl,-rpath," + os.path.join(ROOT, "oracle")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_exprem_gpu_and_gfunc_gpu_through_the_reference_loop(tmp_path):
    d = str(tmp_path)
    N = _write_problem(d, 0.005, [0.0025, 0.005])
    exe = _build_driver(d)
    for par in ("0", "1", "2"):
        env = dict(os.environ, parallel=par, OMP_NUM_THREADS="4")
        r = subprocess.run([exe, d], capture_output=True, text=True, env=env, timeout=600)
        assert r.returncode == 0, (par, r.stdout[-2000:], r.stderr[-2000:])
        assert "N: %d" % N in r.stdout
    read = lambda name: open(os.path.join(d, name), "rb").read()
    stats = {p: open(os.path.join(d, "statistics_%s.txt" % p)).read().splitlines() for p in "012"}
    assert len(stats["2"]) > 5
    assert stats["2"][-1].split()[1] == "5.00000000000000010e-03"
    for p in ("0", "1"):
        assert read("g_%s.bin" % p) == read("g_2.bin")
        assert stats[p] == stats["2"]
        assert read("solution_%s.bin" % p) == read("solution_2.bin")
    sol = np.fromfile(os.path.join(d, "solution_2.bin"))
    assert sol.size == 3 * N and np.all(np.isfinite(sol))
