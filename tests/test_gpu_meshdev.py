"""Macro-mesh preprocessing on the GPU (tsr_macro_mesh_build_device, the
step src/macro_mesh_properties.cpp:241-456 does on the host) against the
host builder (tsr_macro_mesh_build, itself pinned against the reference's
own code in tests/test_mesh_ref.py): every array bit for bit, on the
benchmark's triangle mesh, a quadrilateral mesh with jittered nodes, and
the error for a degenerate element."""
import ctypes as C

import numpy as np
import pytest

from twoscalerich_gb300 import capi
from twoscalerich_gb300 import meshgen

pytestmark = pytest.mark.gpu

FIELDS = [("shape_funcs", lambda nv, Mn, Ne: nv * nv * Ne), ("normals", lambda nv, Mn, Ne: 2 * nv * Ne),
          ("boundary_edge_midpts", lambda nv, Mn, Ne: 4 * nv * Ne),
          ("boundary_edge_normals", lambda nv, Mn, Ne: 4 * nv * Ne),
          ("boundary_edge_lens", lambda nv, Mn, Ne: 2 * nv * Ne), ("CV_area", lambda nv, Mn, Ne: Mn),
          ("SCV_area", lambda nv, Mn, Ne: nv * Ne), ("midx", lambda nv, Mn, Ne: nv * Ne),
          ("midy", lambda nv, Mn, Ne: nv * Ne), ("centroid_elements", lambda nv, Mn, Ne: 2 * Ne),
          ("nodes", lambda nv, Mn, Ne: 2 * Mn)]


def _both(mesh, bc):
    lib = capi.load()
    bc = np.ascontiguousarray(bc, dtype=np.int32)
    out = []
    for f in (lib.tsr_macro_mesh_build, lib.tsr_macro_mesh_build_device):
        m = capi.MacroMesh()
        rc = f(mesh.nv, mesh.n_nodes, capi.ptr(mesh.xy), mesh.n_elems, capi.ptr(mesh.elems),
               mesh.bedges.size // 3, capi.ptr(mesh.bedges), capi.ptr(bc), C.byref(m))
        out.append((rc, m))
    return lib, out


def _compare(mesh, bc):
    lib, ((ra, a), (rb, b)) = _both(mesh, bc)
    assert ra == 0 and rb == 0
    nv, Mn, Ne = a.no_verts, a.no_nodes, a.no_elements
    assert (b.no_verts, b.no_nodes, b.no_elements) == (nv, Mn, Ne)
    for name, size in FIELDS:
        n = size(nv, Mn, Ne)
        x = capi.as_array(getattr(a, name), n, np.float64)
        y = capi.as_array(getattr(b, name), n, np.float64)
        assert np.array_equal(x, y), name
    for name in ("elements", "boundary_condition_edges"):
        x = capi.as_array(getattr(a, name), nv * Ne, np.int32)
        y = capi.as_array(getattr(b, name), nv * Ne, np.int32)
        assert np.array_equal(x, y), name
    lib.tsr_macro_mesh_free(C.byref(a))
    lib.tsr_macro_mesh_free(C.byref(b))


def test_device_geometry_triangles_201():
    _compare(meshgen.macro_unit_square(201), [5, 2, 2, 2, 2])


def test_device_geometry_jittered_quads():
    m = meshgen.macro_unit_square(41, quads=True, segment=(0.0, 0.4))
    rng = np.random.default_rng(3)
    xy = m.xy.reshape(2, -1).copy()
    inner = (xy[0] > 0) & (xy[0] < 1) & (xy[1] > 0) & (xy[1] < 1)
    xy[:, inner] += rng.uniform(-0.2, 0.2, size=(2, int(inner.sum()))) / 40
    m.xy = np.ascontiguousarray(xy.ravel())
    _compare(m, [1, 3, 2, 2, 4])


def test_device_geometry_degenerate_element_refused():
    m = meshgen.macro_unit_square(5)
    m.xy = m.xy.copy()
    e0 = m.elems[:3]
    xy = m.xy.reshape(2, -1)
    xy[:, e0[2]] = xy[:, e0[1]]              # two vertices of element 0 coincide
    lib, ((ra, a), (rb, b)) = _both(m, [1, 2, 2, 2, 2])
    assert ra == 5 and rb == 5                # TSR_ERR_ARG from both builders
