"""The oracle's own mesh preprocessing (oracle/tsr_oracle_mesh.c, used by
the CPU arm of the benchmark so that it loads nothing of the GB300 library)
against this library's and against the reference's compiled preprocessing
(golden vectors).  The two restatements use different formulas (closed-form
P1 coefficients and an LU solve against Gauss-Jordan; shoelace against
diagonal areas), so they agree to rounding: 1e-12 of each field's scale,
1e-10 for the interpolant coefficients, whose inversion cancels (constant
terms of small elements far from the origin; bilinear rows)."""
import numpy as np
import pytest

import oracle
from tests.golden import make_golden as MG
from tests.helpers import golden
from twoscalerich_gb300 import capi
from twoscalerich_gb300 import problem as P

TOL = 1e-12


def _fields(s, fields, nv, n, ne):
    return {f: capi.as_array(getattr(s, f), MG.count(code, nv, n, ne), dt) for f, code, dt in fields}


def _close(a, b, f, tol=TOL):
    if a.dtype.kind == "i":
        assert np.array_equal(a, b), f
        return
    scale = max(np.max(np.abs(b)), 1e-300)
    assert np.max(np.abs(a - b)) <= tol * scale, (f, np.max(np.abs(a - b)) / scale)


@pytest.mark.parametrize("make", [lambda lib: P.config1(lib=lib),
                                  lambda lib: P.config2(n_macro=11, n_micro=7, lib=lib),
                                  lambda lib: P.fixture10(lib=lib),
                                  lambda lib: P.config3(n_macro=9, lib=lib)],
                         ids=["config1", "config2_small", "fixture10_quads", "config3_templates"])
def test_oracle_geometry_matches_library(make):
    a, b = make(None), make(oracle.MeshLib())
    nv = a.macro.no_verts
    fa = _fields(a.macro, MG.MACRO_FIELDS, nv, a.Mn, a.Ne)
    fb = _fields(b.macro, MG.MACRO_FIELDS, nv, b.Mn, b.Ne)
    for f in fa:
        _close(fb[f], fa[f], f, 1e-10 if f == "shape_funcs" else TOL)
    tpl_a = a._tpl if a._tpl is not None else [a.micro]
    tpl_b = b._tpl if b._tpl is not None else [b.micro]
    for ma, mb in zip(tpl_a, tpl_b):
        ga = _fields(ma, MG.MICRO_FIELDS, 3, ma.no_nodes, ma.no_elements)
        gb = _fields(mb, MG.MICRO_FIELDS, 3, mb.no_nodes, mb.no_elements)
        for f in ga:
            _close(gb[f], ga[f], f, 1e-10 if f == "shape_funcs" else TOL)
        assert mb.cell_area == ma.cell_area
    oa, ob = a.options, b.options
    assert [getattr(oa, f) for f, _ in capi.ExpremOptions._fields_] == \
        [getattr(ob, f) for f, _ in capi.ExpremOptions._fields_]


@pytest.mark.parametrize("case", range(len(MG.golden_meshes())))
def test_oracle_geometry_matches_reference_golden(case):
    g = golden()
    name, macro, micro, bc = MG.golden_meshes()[case]
    lib = oracle.load()
    M, m = capi.MacroMesh(), capi.MicroMesh()
    bcs = np.array(bc, dtype=np.int32)
    assert lib.oracle_macro_mesh_build(macro.nv, macro.n_nodes, capi.ptr(macro.xy), macro.n_elems,
                                       capi.ptr(macro.elems), macro.bedges.size // 3,
                                       capi.ptr(macro.bedges), capi.ptr(bcs), M) == 0
    assert lib.oracle_micro_mesh_build(micro.cell[0], micro.cell[1], 3, micro.n_nodes,
                                       capi.ptr(micro.xy), micro.n_elems, capi.ptr(micro.elems),
                                       micro.bedges.size // 3, capi.ptr(micro.bedges), m) == 0
    for mesh, fields, key, nv in ((M, MG.MACRO_FIELDS, "macro", M.no_verts),
                                  (m, MG.MICRO_FIELDS, "micro", 3)):
        ours = _fields(mesh, fields, nv, mesh.no_nodes, mesh.no_elements)
        for f in ours:
            ref = g["%s/%s/%s" % (name, key, f)]
            if f in ("CV_area", "SCV_area") and nv == 3:
                ref = 2.0 * ref          # median-dual thirds (the reference forms sixths)
            _close(ours[f], ref, f, 1e-10 if f == "shape_funcs" else TOL)
    lib.oracle_macro_mesh_free(M)
    lib.oracle_micro_mesh_free(m)
