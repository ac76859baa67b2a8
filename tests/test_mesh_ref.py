"""This library's mesh preprocessing, Keff reader, option defaults and
solution calibration against the reference's own code (golden vectors made
by tests/golden/make_golden.py from the reference's compiled sources, and a
live comparison where the reference tree is present).

Deliberate difference (recorded): triangle SCV / CV / element areas are the
median-dual values, twice the reference's (its second SCV diagonal is
mid_j - mid_{j+1}, src/macro_mesh_properties.cpp:276-279)."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

import oracle
from tests.helpers import golden, reference_root
from tests.golden import make_golden as MG
from twoscalerich_gb300 import capi

AREA_FIELDS = ("CV_area", "SCV_area")


def _ours(macro, micro, bc):
    lib = capi.load()
    M, m = capi.MacroMesh(), capi.MicroMesh()
    bcs = np.array(bc, dtype=np.int32)
    capi.check(lib.tsr_macro_mesh_build(macro.nv, macro.n_nodes, capi.ptr(macro.xy), macro.n_elems,
                                        capi.ptr(macro.elems), macro.bedges.size // 3,
                                        capi.ptr(macro.bedges), capi.ptr(bcs), C.byref(M)), "macro")
    capi.check(lib.tsr_micro_mesh_build(micro.cell[0], micro.cell[1], 3, micro.n_nodes,
                                        capi.ptr(micro.xy), micro.n_elems, capi.ptr(micro.elems),
                                        micro.bedges.size // 3, capi.ptr(micro.bedges),
                                        C.byref(m)), "micro")
    return M, m


def _compare(ours, ref_arrays, fields, tri):
    nv = ours.no_verts
    Mn, Ne = ours.no_nodes, ours.no_elements
    for f, code, dt in fields:
        a = capi.as_array(getattr(ours, f), MG.count(code, nv, Mn, Ne), dt)
        b = ref_arrays[f]
        if dt == np.int32:
            assert np.array_equal(a, b), f
            continue
        if f in AREA_FIELDS and tri:
            b = 2.0 * b
        scale = max(np.max(np.abs(b)), 1e-300)
        # bilinear coefficients come from inverting [x y xy 1], whose
        # condition number is ~1e4 for 0.1 m quads near (1, 1): two correct
        # inversions (the reference's closed form, Gauss-Jordan here) differ
        # at eps * cond
        tol = 1e-10 if (f == "shape_funcs" and nv == 4) else 1e-12
        assert np.max(np.abs(a - b)) <= tol * scale, (f, np.max(np.abs(a - b)), scale)


@pytest.mark.parametrize("case", range(len(MG.golden_meshes())))
def test_geometry_matches_reference_golden(case):
    g = golden()
    name, macro, micro, bc = MG.golden_meshes()[case]
    M, m = _ours(macro, micro, bc)
    ref_M = {f: g["%s/macro/%s" % (name, f)] for f, _, _ in MG.MACRO_FIELDS}
    ref_m = {f: g["%s/micro/%s" % (name, f)] for f, _, _ in MG.MICRO_FIELDS}
    _compare(M, ref_M, MG.MACRO_FIELDS, tri=(M.no_verts == 3))
    _compare(m, ref_m, MG.MICRO_FIELDS, tri=True)
    # the reference reads the cell size as long double and multiplies there
    # (src/micro_mesh_properties.cpp:54-57, 194): equal to 1 ulp
    assert abs(m.cell_area - g["%s/micro/cell_area" % name][0]) <= np.spacing(m.cell_area)
    # micro element areas: the median-dual SCVs sum to the element area
    ea = capi.as_array(m.element_area, m.no_elements)
    assert abs(ea.sum() - capi.as_array(m.CV_area, m.no_nodes).sum()) < 1e-15


@pytest.mark.parametrize("case", range(len(MG.golden_meshes())))
def test_micro_boundary_calibration_matches_reference_writer(case):
    """src/save_solution.cpp's calibration of the micro boundary unknowns is
    the interpolant the cell kernels use."""
    g = golden()
    name, macro, micro, bc = MG.golden_meshes()[case]
    M, m = _ours(macro, micro, bc)
    ud = capi.UserData()
    ud.macro_mesh, ud.micro_mesh, ud.model_type = M, m, 3
    N = M.no_nodes + M.no_elements * m.no_nodes
    u = MG.solution_state(N)
    assert np.array_equal(u[:8], g["%s/solution/u_check" % name])
    capi.check(capi.load().tsr_calibrate_micro_boundary(C.byref(ud), None, capi.ptr(u)), "calibrate")
    idx = g["%s/solution/index" % name]
    ref = g["%s/solution/value" % name]
    # quadrilateral interpolants inherit the conditioning of their coefficients
    tol = 1e-13 if M.no_verts == 3 else 1e-10
    assert np.max(np.abs(u[idx] - ref)) <= tol * np.max(np.abs(ref))
    # and nothing else changed
    untouched = np.setdiff1d(np.arange(N), idx)
    assert np.array_equal(u[untouched], MG.solution_state(N)[untouched])


def test_keff_reader_matches_reference_golden():
    g = golden()
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "Keff.txt")
        open(f, "wb").write(g["keff/text"].tobytes())
        K = capi.Keff()
        capi.check(capi.load().tsr_read_effective_conductivity(f.encode(), C.byref(K)), "keff")
        hdr = g["keff/header"]
        assert (K.epsilonA, K.no_hvalues, K.logr, K.logh_first) == tuple(hdr.tolist()[:1]) + (int(hdr[1]),) + tuple(hdr.tolist()[2:])
        assert np.array_equal(capi.as_array(K.logh_values, K.no_hvalues), g["keff/logh"])
        assert np.array_equal(capi.as_array(K.Keff_values, 4 * K.no_hvalues), g["keff/values"])
        capi.load().tsr_keff_free(C.byref(K))


def test_options_defaults_match_reference():
    o = capi.ExpremOptions()
    capi.check(capi.load().tsr_set_exprem_options(C.byref(o)), "options")
    ours = np.array([getattr(o, f) for f, _ in capi.ExpremOptions._fields_], dtype=float)
    assert np.array_equal(ours, golden()["options"])


def test_missing_files_return_io_error():
    lib = capi.load()
    M = capi.MacroMesh()
    bc = np.array([1, 2, 2, 2, 2], dtype=np.int32)
    assert lib.tsr_macro_mesh_properties(b"/nonexistent.msh", C.byref(M), capi.ptr(bc)) == 11
    assert lib.tsr_micro_mesh_properties(b"/nonexistent.msh", C.byref(capi.MicroMesh())) == 11
    assert lib.tsr_read_effective_conductivity(b"/nonexistent.txt", C.byref(capi.Keff())) == 11


def test_bad_element_indices_rejected():
    lib = capi.load()
    xy = np.array([0, 1, 0, 0, 0, 1], dtype=float)
    el = np.array([0, 1, 7], dtype=np.int32)
    bc = np.array([2, 2, 2, 2, 2], dtype=np.int32)
    rc = lib.tsr_macro_mesh_build(3, 3, capi.ptr(xy), 1, capi.ptr(el), 0, None, capi.ptr(bc),
                                  C.byref(capi.MacroMesh()))
    assert rc == 5


@pytest.mark.skipif(reference_root() is None or oracle.load_ref() is None,
                    reason="reference tree / oracle/_ref not present")
@pytest.mark.parametrize("pair", [("macro_structured_10by10.msh", "microB_unstructured_10by10.msh"),
                                  ("macro_structured_20by20.msh", "microB_unstructured_20by20.msh")])
def test_reference_fixture_meshes_live(pair):
    """The reference's own test meshes through both preprocessors."""
    ref = oracle.load_ref()
    lib = capi.load()
    d = os.path.join(reference_root(), "tests", "Richards_Equation")
    bc = np.array([1, 3, 2, 2, 2], dtype=np.int32)        # src/main.cpp:180-184
    fmac, fmic = (os.path.join(d, f).encode() for f in pair)
    Mr, Mo = capi.MacroMesh(), capi.MacroMesh()
    assert ref.ref_macro_mesh_properties(fmac, C.byref(Mr), capi.ptr(bc)) == 0
    capi.check(lib.tsr_macro_mesh_properties(fmac, C.byref(Mo), capi.ptr(bc)), "macro")
    mr, mo = capi.MicroMesh(), capi.MicroMesh()
    assert ref.ref_micro_mesh_properties(fmic, C.byref(mr)) == 0
    capi.check(lib.tsr_micro_mesh_properties(fmic, C.byref(mo)), "micro")
    ref_M = MG.extract(Mr, MG.MACRO_FIELDS, Mr.no_verts, Mr.no_nodes, Mr.no_elements)
    ref_m = MG.extract(mr, MG.MICRO_FIELDS, mr.no_verts, mr.no_nodes, mr.no_elements)
    _compare(Mo, ref_M, MG.MACRO_FIELDS, tri=(Mo.no_verts == 3))
    _compare(mo, ref_m, MG.MICRO_FIELDS, tri=True)
    assert abs(capi.as_array(Mo.CV_area, Mo.no_nodes).sum() - 1.0) < 1e-12


def test_reference_fixture_through_library_readers(tmp_path):
    """The reference's own scenario (its problem_options.txt, 10x10
    quadrilateral mesh, 167-node inclusion mesh and Keff table, kept in
    tests/golden/ref_fixture.npz) assembled by this library's readers the
    way the reference's main() assembles it: same geometry as the
    reference's own preprocessing, same Keff table, and the driver's
    boundary_flux quirk (18 values for 19 reads: boundary_flux = 1.89)."""
    from tests.helpers import FIXTURE, write_reference_fixture
    from twoscalerich_gb300 import problem as P
    g = np.load(FIXTURE)
    p = P.from_reference_files(write_reference_fixture(str(tmp_path)))
    assert p.ud.boundary_flux == 1.89 == g["options/boundary_flux"][0]
    assert p.u0[0] == -20.0 and p.tend == 2.0 and list(p.tspan) == [2.0, 1.0, 2.0]
    assert p.N == 121 + 100 * 167
    ref_M = {f: g["refgeom/macro/%s" % f] for f, _, _ in MG.MACRO_FIELDS}
    ref_m = {f: g["refgeom/micro/%s" % f] for f, _, _ in MG.MICRO_FIELDS}
    _compare(p.macro, ref_M, MG.MACRO_FIELDS, tri=False)
    _compare(p.micro, ref_m, MG.MICRO_FIELDS, tri=True)
    assert abs(p.micro.cell_area - g["refgeom/micro/cell_area"][0]) <= np.spacing(p.micro.cell_area)
    K = p.keff
    assert (K.epsilonA, K.no_hvalues, K.logr, K.logh_first) == (
        g["keff/header"][0], int(g["keff/header"][1]), g["keff/header"][2], g["keff/header"][3])
    assert np.array_equal(capi.as_array(K.Keff_values, 4 * K.no_hvalues), g["keff/values"])
    p.close()


def test_reference_fixture_calibration_matches_reference_writer(tmp_path):
    """save_solution's micro-boundary calibration (src/save_solution.cpp:41-102)
    of the reference's own scenario, on the geometry this library reads."""
    from tests.helpers import FIXTURE, write_reference_fixture
    from twoscalerich_gb300 import problem as P
    g = np.load(FIXTURE)
    p = P.from_reference_files(write_reference_fixture(str(tmp_path)))
    u = MG.solution_state(p.N)
    assert np.array_equal(u[:8], g["solution/u_check"])
    capi.check(capi.load().tsr_calibrate_micro_boundary(C.byref(p.ud), None, capi.ptr(u)), "calibrate")
    idx, ref = g["solution/index"], g["solution/value"]
    assert np.max(np.abs(u[idx] - ref)) <= 1e-10 * np.max(np.abs(ref))
    untouched = np.setdiff1d(np.arange(p.N), idx)
    assert np.array_equal(u[untouched], MG.solution_state(p.N)[untouched])
    p.close()


def test_solution_writer_matches_reference_layout(tmp_path):
    """tsr_save_solution (the reference's save_solution: calibrate the
    stored rows in place, then write them) on the reference's own scenario
    read by this library: the same file layout as the reference's writer,
    the same calibrated values as its golden output (1e-10, the interpolant
    formulas differ in rounding), every other value exactly."""
    from tests.helpers import FIXTURE, write_reference_fixture
    from twoscalerich_gb300 import problem as P
    g = np.load(FIXTURE)
    p = P.from_reference_files(write_reference_fixture(str(tmp_path)))
    u = MG.solution_state(p.N)
    rows = np.concatenate([u, u + 1.0])          # two rows: t = 0 and t = tspan[1]
    tspan = np.array([1.0, 0.25])
    path = str(tmp_path / "solution.txt")
    capi.check(capi.load().tsr_save_solution(path.encode(), capi.ptr(tspan), capi.ptr(rows), 1,
                                             C.byref(p.ud)), "tsr_save_solution")
    text = open(path).read()
    lines = text.splitlines()
    assert lines[0] == "2" and len(lines) == 3
    tok0, tok1 = lines[1].split(" "), lines[2].split(" ")
    assert tok0[0] == "0.00000000000000000000e+00" and tok1[0] == "%.20e" % 0.25
    assert len(tok0) == p.N + 1
    written = np.array(tok0[1:], dtype=float)
    assert np.array_equal(written, rows[:p.N])       # in place, then written exactly
    idx, ref = g["solution/index"], g["solution/value"]
    assert np.max(np.abs(written[idx] - ref)) <= 1e-10 * np.max(np.abs(ref))
    untouched = np.setdiff1d(np.arange(p.N), idx)
    assert np.array_equal(written[untouched], u[untouched])
    p.close()


@pytest.mark.skipif(oracle.load_ref() is None, reason="oracle/_ref not present")
def test_solution_writer_bytes_match_reference_writer(tmp_path):
    """Byte for byte against the reference's own save_solution (compiled in
    oracle/_ref) on rows whose micro-boundary entries are already calibrated
    (so both writers see the same values)."""
    ref = oracle.load_ref()
    name, macro, micro, bc = MG.golden_meshes()[0]
    M, m = _ours(macro, micro, bc)
    ud = capi.UserData()
    ud.macro_mesh, ud.micro_mesh, ud.model_type = M, m, 3
    N = M.no_nodes + M.no_elements * m.no_nodes
    ud.N = N
    u = MG.solution_state(N)
    capi.check(capi.load().tsr_calibrate_micro_boundary(C.byref(ud), None, capi.ptr(u)), "calibrate")
    tspan = np.array([0.0])
    ours, theirs = str(tmp_path / "ours.txt"), str(tmp_path / "ref.txt")
    capi.check(capi.load().tsr_save_solution(ours.encode(), capi.ptr(tspan), capi.ptr(u.copy()), 0,
                                             C.byref(ud)), "save")
    # the reference's writer calibrates again with its own interpolant
    # formula: the micro-boundary entries may differ in the last bits, every
    # other token must be the same text
    ref.ref_save_solution(theirs.encode(), capi.ptr(tspan), capi.ptr(u.copy()), 0, C.byref(ud))
    a, b = open(ours).read().split(), open(theirs).read().split()
    assert len(a) == len(b) == N + 2 and a[0] == b[0] == "1" and a[1] == b[1]
    bnd = np.zeros(N, bool)
    mb = capi.as_array(m.boundary_nodes, m.no_nodes, np.int32) == 1
    for k in range(M.no_elements):
        bnd[M.no_nodes + k * m.no_nodes:M.no_nodes + (k + 1) * m.no_nodes] = mb
    assert all(a[2 + i] == b[2 + i] for i in np.nonzero(~bnd)[0])
    va, vb = np.array(a[2:], dtype=float), np.array(b[2:], dtype=float)
    assert np.max(np.abs(va - vb)) <= 1e-13 * np.max(np.abs(vb))
