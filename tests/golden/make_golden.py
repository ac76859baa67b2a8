"""Generate the golden vectors of tests/golden/ref_golden.npz by running the
reference's OWN code (its src/phipade.cpp, src/macro_mesh_properties.cpp,
src/micro_mesh_properties.cpp, src/read_effective_conductivity.cpp,
src/save_solution.cpp and src/set_exprem_options.cpp, compiled from the
reference tree by `make -C oracle ref` into oracle/_ref/libtsr_ref.so) on
seeded inputs that this script builds itself:

  * meshes from twoscalerich_gb300.meshgen, written in the reference's text
    format: the 21x21 triangulated macro mesh and 11x11 inclusion of the
    21x21 configuration, the 11x11-node quadrilateral macro mesh and the
    irregular inclusion of the 10x10 fixture shape;
  * upper Hessenberg matrices (seed 20261203) for phipade, m = 1..30,
    several alpha;
  * a Keff table in the reference's format;
  * one state vector per mesh pair for the solution writer's calibration.

Run (where the reference tree is present):
    make -C oracle ref && python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from twoscalerich_gb300 import capi, meshgen  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "ref_golden.npz")
MAXK = 40

MACRO_FIELDS = [("elements", "nvNe", np.int32), ("nodes", "2Mn", np.float64),
                ("shape_funcs", "nv2Ne", np.float64), ("normals", "2nvNe", np.float64),
                ("boundary_edge_midpts", "4nvNe", np.float64),
                ("boundary_edge_normals", "4nvNe", np.float64),
                ("boundary_edge_lens", "2nvNe", np.float64),
                ("boundary_condition_edges", "nvNe", np.int32), ("CV_area", "Mn", np.float64),
                ("SCV_area", "nvNe", np.float64), ("midx", "nvNe", np.float64),
                ("midy", "nvNe", np.float64), ("centroid_elements", "2Ne", np.float64)]
MICRO_FIELDS = [("elements", "nvNe", np.int32), ("boundary_nodes", "Mn", np.int32),
                ("nodes", "2Mn", np.float64), ("shape_funcs", "nv2Ne", np.float64),
                ("normals", "2nvNe", np.float64), ("boundary_edges", "nvNe", np.int32),
                ("boundary_edge_midpts", "4nvNe", np.float64),
                ("boundary_edge_normals", "4nvNe", np.float64),
                ("boundary_edge_lens", "2nvNe", np.float64),
                ("centroid_elements", "2Ne", np.float64), ("CV_area", "Mn", np.float64),
                ("midx", "nvNe", np.float64), ("midy", "nvNe", np.float64),
                ("vectors", "2Mn", np.float64)]


def count(code, nv, Mn, Ne):
    return {"nvNe": nv * Ne, "2Mn": 2 * Mn, "nv2Ne": nv * nv * Ne, "2nvNe": 2 * nv * Ne,
            "4nvNe": 4 * nv * Ne, "Mn": Mn, "2Ne": 2 * Ne}[code]


def extract(s, fields, nv, Mn, Ne):
    return {f: capi.as_array(getattr(s, f), count(code, nv, Mn, Ne), dt) for f, code, dt in fields}


def golden_meshes():
    """(name, macro Mesh, micro Mesh, macro_bc) built by this project's generator."""
    return [
        ("config1", meshgen.macro_unit_square(21), meshgen.micro_square_inclusion(11, cell=0.05, side=0.5),
         [5, 2, 2, 2, 2]),
        ("fixture10", meshgen.macro_unit_square(11, quads=True, segment=(0.0, 0.4)),
         meshgen.micro_square_inclusion(11, cell=0.1, side=0.6, jitter=0.25, seed=20261203),
         [1, 3, 2, 2, 2]),
    ]


def solution_state(N):
    """The state the solution-writer golden is generated from (seed 11)."""
    return -5.0 + np.random.default_rng(11).normal(0, 0.5, N)


def hessenberg_cases():
    rng = np.random.default_rng(20261203)
    cases = []
    for m in list(range(1, 13)) + [16, 20, 25, 30]:
        for alpha in (1e-3, 0.7, 3.0, 40.0):
            H = np.zeros((MAXK, MAXK + 1))            # column major, ld = MAXK + 1
            for j in range(m):
                for i in range(min(j + 2, m + 1)):
                    H[j, i] = rng.normal() * (2.0 if i == j else 1.0) - (3.0 if i == j else 0.0)
            cases.append((m, alpha, H))
    return cases


def main():
    ref = oracle.load_ref()
    if ref is None:
        raise SystemExit("oracle/_ref/libtsr_ref.so missing: run make -C oracle ref")
    out = {}
    tmp = tempfile.mkdtemp()
    for name, macro, micro, bc in golden_meshes():
        fmac = os.path.join(tmp, name + "_macro.msh")
        fmic = os.path.join(tmp, name + "_micro.msh")
        macro.write(fmac)
        micro.write(fmic)
        M = capi.MacroMesh()
        bcs = np.array(bc, dtype=np.int32)
        assert ref.ref_macro_mesh_properties(fmac.encode(), C.byref(M), capi.ptr(bcs)) == 0
        for k, v in extract(M, MACRO_FIELDS, M.no_verts, M.no_nodes, M.no_elements).items():
            out["%s/macro/%s" % (name, k)] = v
        m = capi.MicroMesh()
        assert ref.ref_micro_mesh_properties(fmic.encode(), C.byref(m)) == 0
        for k, v in extract(m, MICRO_FIELDS, m.no_verts, m.no_nodes, m.no_elements).items():
            out["%s/micro/%s" % (name, k)] = v
        out["%s/micro/cell_area" % name] = np.array([m.cell_area])
        # the solution writer's calibration of the micro boundary unknowns
        ud = capi.UserData()
        ud.macro_mesh, ud.micro_mesh = M, m
        ud.model_type = 3
        N = M.no_nodes + M.no_elements * m.no_nodes
        ud.N = N
        u = solution_state(N)
        tspan = np.array([0.0])
        fsol = os.path.join(tmp, name + "_sol.txt")
        ref.ref_save_solution(fsol.encode(), capi.ptr(tspan), capi.ptr(u.copy()), 0, C.byref(ud))
        row = np.array(open(fsol).read().split()[1:], dtype=float)   # skip the count line
        written = row[1:]                                            # skip the time column
        changed = np.nonzero(written != u)[0]
        # u is regenerated by the tests from the same seed; keep only the
        # calibrated (micro-boundary) entries of the written row
        out["%s/solution/index" % name] = changed.astype(np.int64)
        out["%s/solution/value" % name] = written[changed]
        out["%s/solution/u_check" % name] = u[:8]
    # phipade
    # stored compactly: H(1:m+1, 1:m) and phi(1:m, 1:m) of each case, column
    # major, concatenated
    Hs, outs, ms, alphas = [], [], [], []
    for m, alpha, H in hessenberg_cases():
        phi = np.zeros((MAXK, MAXK))
        Hc = np.ascontiguousarray(H)
        ref.ref_phipade(capi.ptr(phi.ravel()), capi.ptr(Hc.ravel()), alpha, m, MAXK)
        Hs.append(H[:m, :m + 1].ravel())
        outs.append(phi[:m, :m].ravel())
        ms.append(m)
        alphas.append(alpha)
    out["phipade/H"] = np.concatenate(Hs)
    out["phipade/phi"] = np.concatenate(outs)
    out["phipade/m"] = np.array(ms)
    out["phipade/alpha"] = np.array(alphas)
    # Keff reader on a table in the reference's format
    fk = os.path.join(tmp, "Keff.txt")
    logh = 1.3 - 0.0333 * np.arange(40)
    rows = np.stack([logh, 0.02 / (1 + 10 ** logh), -1e-4 * np.ones(40), -1e-4 * np.ones(40),
                     0.015 / (1 + 10 ** logh)], 1)
    with open(fk, "w") as f:
        f.write("0.6\n40\n-0.0333\n1.3\n")
        for r in rows:
            f.write(" ".join("%.15e" % v for v in r) + "\n")
    K = capi.Keff()
    assert ref.ref_read_effective_conductivity(fk.encode(), C.byref(K)) == 0
    out["keff/text"] = np.frombuffer(open(fk, "rb").read(), dtype=np.uint8)
    out["keff/header"] = np.array([K.epsilonA, K.no_hvalues, K.logr, K.logh_first])
    out["keff/logh"] = capi.as_array(K.logh_values, K.no_hvalues)
    out["keff/values"] = capi.as_array(K.Keff_values, 4 * K.no_hvalues)
    o = capi.ExpremOptions()
    ref.ref_set_exprem_options(C.byref(o))
    out["options"] = np.array([getattr(o, f) for f, _ in capi.ExpremOptions._fields_], dtype=float)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    main()
