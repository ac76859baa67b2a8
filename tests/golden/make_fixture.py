"""Generate tests/golden/ref_fixture.npz from the reference's OWN test
scenario (tests/Richards_Equation of the reference tree): the 10x10
quadrilateral macro mesh, the 167-node unstructured inclusion mesh, the
tabulated Keff(h) tensor and the problem options, together with what the
reference's own code (compiled by `make -C oracle ref` into
oracle/_ref/libtsr_ref.so) computes from them:

  * mesh/...      the raw contents of the two mesh files (node coordinates,
                  boundary edges with tags, elements; 0-based), so that the
                  GPU tests can write the files again where the reference
                  tree is absent and read them with this library's readers;
  * keff/...      the Keff table file as read by the reference's reader;
  * options/...   problem_options.txt read the way src/main.cpp:32-146 reads
                  it -- including its quirk: the file holds 18 values for 19
                  reads, so the last fscanf fails and boundary_flux keeps the
                  previous value, 1.89;
  * refgeom/...   the macro and micro geometry from the reference's
                  macro_mesh_properties / micro_mesh_properties (the arrays
                  a reference-built user_data carries);
  * solution/...  the reference's save_solution calibration of a seeded
                  state on that geometry.

Run (where the reference tree is present):
    make -C oracle ref && python tests/golden/make_fixture.py
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from tests.golden import make_golden as MG  # noqa: E402
from tests.helpers import reference_root  # noqa: E402
from twoscalerich_gb300 import capi  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "ref_fixture.npz")
MACRO_FILE = "macro_structured_10by10.msh"
MICRO_FILE = "microB_unstructured_10by10.msh"
MACRO_BC = [1, 3, 2, 2, 2]          # src/main.cpp:180-184


def read_mesh_text(path, micro):
    """The reference mesh text format (src/macro_mesh_properties.cpp:56-136,
    src/micro_mesh_properties.cpp:56-140) as arrays: (cell, nv, xy, bedges,
    elems), 0-based node numbers."""
    tok = open(path).read().split()
    pos = 0
    cell = None
    if micro:
        cell = np.array([float(tok[0]), float(tok[1])])
        pos = 2
    nv, n = int(tok[pos]), int(tok[pos + 1])
    pos += 2
    xy = np.array(tok[pos:pos + 2 * n], dtype=float).reshape(n, 2)
    pos += 2 * n
    nb = int(tok[pos])
    pos += 1
    b = np.array(tok[pos:pos + 3 * nb], dtype=np.int64).reshape(nb, 3)
    pos += 3 * nb
    ne = int(tok[pos])
    pos += 1
    el = np.array(tok[pos:pos + nv * ne], dtype=np.int64).reshape(ne, nv)
    b[:, :2] -= 1
    return (cell, nv, np.concatenate([xy[:, 0], xy[:, 1]]), b.astype(np.int32).ravel(),
            (el - 1).astype(np.int32).ravel())


def read_options(path):
    """problem_options.txt as src/main.cpp:32-146 reads it: three file names,
    h0, tend, no_solns, no_solns times, soil A (Ksat, thetar, thetas, alpha,
    n), soil B, boundary_flux -- a missing value keeps the previous one."""
    tok = open(path).read().split()
    vals = tok[3:]
    pos = 0
    last = [0.0]

    def num():
        nonlocal pos
        if pos < len(vals):
            last[0] = float(vals[pos])
        pos += 1
        return last[0]
    h0 = num()
    tend = num()
    no_solns = int(num())
    tspan = [num() for _ in range(no_solns)]
    soilA = [num() for _ in range(5)]
    soilB = [num() for _ in range(5)]
    bflux = num()
    return dict(h0=h0, tend=tend, tspan=np.array(tspan), soilA=np.array(soilA),
                soilB=np.array(soilB), boundary_flux=bflux, tokens=len(vals))


def main():
    ref = oracle.load_ref()
    root = reference_root()
    if ref is None or root is None:
        raise SystemExit("reference tree or oracle/_ref/libtsr_ref.so missing: run make -C oracle ref")
    d = os.path.join(root, "tests", "Richards_Equation")
    out = {}
    for name, f, micro in (("macro", MACRO_FILE, False), ("micro", MICRO_FILE, True)):
        cell, nv, xy, bedges, elems = read_mesh_text(os.path.join(d, f), micro)
        out["mesh/%s/nv" % name] = np.array([nv])
        out["mesh/%s/xy" % name] = xy
        out["mesh/%s/bedges" % name] = bedges
        out["mesh/%s/elems" % name] = elems
        if micro:
            out["mesh/micro/cell"] = cell
    K = capi.Keff()
    assert ref.ref_read_effective_conductivity(os.path.join(d, "Keff.txt").encode(), C.byref(K)) == 0
    out["keff/header"] = np.array([K.epsilonA, K.no_hvalues, K.logr, K.logh_first])
    out["keff/logh"] = capi.as_array(K.logh_values, K.no_hvalues).copy()
    out["keff/values"] = capi.as_array(K.Keff_values, 4 * K.no_hvalues).copy()
    opt = read_options(os.path.join(d, "problem_options.txt"))
    for k, v in opt.items():
        out["options/%s" % k] = np.atleast_1d(np.asarray(v, dtype=float))
    bcs = np.array(MACRO_BC, dtype=np.int32)
    M = capi.MacroMesh()
    assert ref.ref_macro_mesh_properties(os.path.join(d, MACRO_FILE).encode(), C.byref(M), capi.ptr(bcs)) == 0
    for k, v in MG.extract(M, MG.MACRO_FIELDS, M.no_verts, M.no_nodes, M.no_elements).items():
        out["refgeom/macro/%s" % k] = v.copy()
    out["refgeom/macro/counts"] = np.array([M.no_verts, M.no_nodes, M.no_elements])
    m = capi.MicroMesh()
    assert ref.ref_micro_mesh_properties(os.path.join(d, MICRO_FILE).encode(), C.byref(m)) == 0
    for k, v in MG.extract(m, MG.MICRO_FIELDS, m.no_verts, m.no_nodes, m.no_elements).items():
        out["refgeom/micro/%s" % k] = v.copy()
    out["refgeom/micro/counts"] = np.array([m.no_verts, m.no_nodes, m.no_elements])
    out["refgeom/micro/cell_area"] = np.array([m.cell_area])
    # the solution writer's calibration on the reference-built geometry
    ud = capi.UserData()
    ud.macro_mesh, ud.micro_mesh = M, m
    ud.model_type = 3
    N = M.no_nodes + M.no_elements * m.no_nodes
    ud.N = N
    u = MG.solution_state(N)
    tmp = tempfile.mkdtemp()
    fsol = os.path.join(tmp, "sol.txt")
    tspan = np.array([0.0])
    ref.ref_save_solution(fsol.encode(), capi.ptr(tspan), capi.ptr(u.copy()), 0, C.byref(ud))
    row = np.array(open(fsol).read().split()[1:], dtype=float)
    written = row[1:]
    changed = np.nonzero(written != u)[0]
    out["solution/index"] = changed.astype(np.int64)
    out["solution/value"] = written[changed]
    out["solution/u_check"] = u[:8]
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    main()
