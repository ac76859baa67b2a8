"""Seeded synthetic meshes in the reference's mesh model.

The reference reads gmsh-derived text meshes (tests/Richards_Equation/*.msh;
format read by src/macro_mesh_properties.cpp:56-136 and
src/micro_mesh_properties.cpp:56-140).  These generators produce the same
content (node coordinates, boundary segments with tags, element connectivity)
directly as arrays for ``tsr_macro_mesh_build`` / ``tsr_micro_mesh_build``,
and can also write it in the reference's text format.

Arrays: xy = [x_0..x_{n-1}, y_0..y_{n-1}]; elems element-major 0-based
(vertex v of element k at k*nv+v, counter-clockwise); bedges rows
(node a, node b, tag) 0-based.  Macro tags follow the reference fixture:
-1 the specified segment on the top side (flux in the reference, Dirichlet in
the configurations built here), -2 south, -3 east, -4 west, -5 rest of the
top side.  Micro tag -1 marks the inclusion boundary.
"""
import numpy as np

SOUTH, EAST, WEST, NORTH_REST, TOP_SEGMENT = -2, -3, -4, -5, -1


class Mesh:
    def __init__(self, nv, xy, elems, bedges, cell=None):
        self.nv = nv
        self.xy = np.ascontiguousarray(xy, dtype=np.float64)
        self.elems = np.ascontiguousarray(elems, dtype=np.int32)
        self.bedges = np.ascontiguousarray(bedges, dtype=np.int32)
        self.cell = cell  # (width, height) for micro meshes

    @property
    def n_nodes(self):
        return self.xy.size // 2

    @property
    def n_elems(self):
        return self.elems.size // self.nv

    def write(self, path):
        """Write the mesh in the reference's text format (1-based)."""
        n = self.n_nodes
        lines = []
        if self.cell is not None:
            lines += ["%.16f" % self.cell[0], "%.16f" % self.cell[1]]
        lines += [str(self.nv), str(n)]
        lines += ["%.16f %.16f" % (self.xy[i], self.xy[n + i]) for i in range(n)]
        b = self.bedges.reshape(-1, 3)
        lines.append(str(len(b)))
        lines += ["%d %d %d" % (r[0] + 1, r[1] + 1, r[2]) for r in b]
        e = self.elems.reshape(-1, self.nv)
        lines.append(str(len(e)))
        lines += [" ".join(str(v + 1) for v in r) for r in e]
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")


def _grid_nodes(nx, ny, x0, y0, w, h):
    xs = x0 + w * np.arange(nx) / (nx - 1)
    ys = y0 + h * np.arange(ny) / (ny - 1)
    X, Y = np.meshgrid(xs, ys)            # node id = j*nx + i
    return np.concatenate([X.ravel(), Y.ravel()])


def _grid_boundary(nx, ny, xy, tag_fn):
    n = nx * ny
    rows = []
    for i in range(nx - 1):                                  # south
        a, b = i, i + 1
        rows.append((a, b, tag_fn("south", 0.5 * (xy[a] + xy[b]), 0.5 * (xy[n + a] + xy[n + b]))))
    for j in range(ny - 1):                                  # east
        a, b = j * nx + nx - 1, (j + 1) * nx + nx - 1
        rows.append((a, b, tag_fn("east", 0.5 * (xy[a] + xy[b]), 0.5 * (xy[n + a] + xy[n + b]))))
    for i in range(nx - 1, 0, -1):                           # north
        a, b = (ny - 1) * nx + i, (ny - 1) * nx + i - 1
        rows.append((a, b, tag_fn("north", 0.5 * (xy[a] + xy[b]), 0.5 * (xy[n + a] + xy[n + b]))))
    for j in range(ny - 1, 0, -1):                           # west
        a, b = j * nx, (j - 1) * nx
        rows.append((a, b, tag_fn("west", 0.5 * (xy[a] + xy[b]), 0.5 * (xy[n + a] + xy[n + b]))))
    return np.array(rows, dtype=np.int32).ravel()


def _grid_tris(nx, ny):
    j, i = np.meshgrid(np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    a = (j * nx + i).ravel()
    b, c, d = a + 1, a + nx + 1, a + nx
    t1 = np.stack([a, b, c], 1)
    t2 = np.stack([a, c, d], 1)
    return np.stack([t1, t2], 1).reshape(-1, 3).ravel()


def _grid_quads(nx, ny):
    j, i = np.meshgrid(np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    a = (j * nx + i).ravel()
    return np.stack([a, a + 1, a + nx + 1, a + nx], 1).ravel()


def macro_tag_fn(segment=(0.0, 1.0)):
    """Tags of the unit-square sides; the top side's part with x in
    `segment` gets tag -1."""
    lo, hi = segment

    def fn(side, xm, ym):
        if side == "south":
            return SOUTH
        if side == "east":
            return EAST
        if side == "west":
            return WEST
        return TOP_SEGMENT if (lo <= xm <= hi) else NORTH_REST
    return fn


def macro_unit_square(n, quads=False, segment=(0.0, 1.0)):
    """n x n nodes on [0,1]^2; two triangles per square (diagonal from the
    lower-left corner) or quadrilaterals."""
    xy = _grid_nodes(n, n, 0.0, 0.0, 1.0, 1.0)
    elems = _grid_quads(n, n) if quads else _grid_tris(n, n)
    bed = _grid_boundary(n, n, xy, macro_tag_fn(segment))
    return Mesh(4 if quads else 3, xy, elems, bed)


def micro_square_inclusion(n, cell=1.0, side=0.5, jitter=0.0, seed=0):
    """A square inclusion of side `side`*cell centred in a cell of width
    `cell`, meshed by an n x n node triangulated grid (the inclusion only:
    material B; the surrounding material A is the macro continuum).  With
    jitter > 0 interior nodes are displaced by up to jitter * spacing,
    giving an irregular triangulation."""
    w = side * cell
    x0 = 0.5 * (cell - w)
    xy = _grid_nodes(n, n, x0, x0, w, w)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        hsp = w / (n - 1)
        nn = n * n
        j, i = np.divmod(np.arange(nn), n)
        interior = (i > 0) & (i < n - 1) & (j > 0) & (j < n - 1)
        d = rng.uniform(-jitter, jitter, size=(2, nn)) * hsp
        xy[:nn][interior] += d[0][interior]
        xy[nn:][interior] += d[1][interior]
    elems = _grid_tris(n, n)
    bed = _grid_boundary(n, n, xy, lambda *a: -1)
    return Mesh(3, xy, elems, bed, cell=(cell, cell))


def read_mesh(path, micro=False):
    """Read a mesh in the reference's text format."""
    tok = open(path).read().split()
    p = 0

    def nxt():
        nonlocal p
        p += 1
        return tok[p - 1]
    cell = None
    if micro:
        cell = (float(nxt()), float(nxt()))
    nv = int(nxt())
    n = int(nxt())
    xy = np.zeros(2 * n)
    for i in range(n):
        xy[i] = float(nxt())
        xy[n + i] = float(nxt())
    nb = int(nxt())
    bed = np.array([int(nxt()) for _ in range(3 * nb)], dtype=np.int64).reshape(-1, 3)
    bed[:, :2] -= 1
    ne = int(nxt())
    el = np.array([int(nxt()) for _ in range(nv * ne)], dtype=np.int64) - 1
    return Mesh(nv, xy, el, bed.ravel(), cell=cell)


def micro_disk_inclusion(n, cell=1.0, diameter=0.5):
    """A disk inclusion of diameter `diameter`*cell centred in the cell,
    meshed by an n x n grid mapped onto the disk (elliptical grid mapping
    (a, b) -> (a sqrt(1 - b^2/2), b sqrt(1 - a^2/2)), orientation
    preserving); the square's boundary maps onto the circle."""
    s = np.linspace(-1.0, 1.0, n)
    A, B = np.meshgrid(s, s)                     # node id = j*n + i
    X = A * np.sqrt(1.0 - B * B / 2.0)
    Y = B * np.sqrt(1.0 - A * A / 2.0)
    r = 0.5 * diameter * cell
    xy = np.concatenate([0.5 * cell + r * X.ravel(), 0.5 * cell + r * Y.ravel()])
    elems = _grid_tris(n, n)
    bed = _grid_boundary(n, n, xy, lambda *a: -1)
    return Mesh(3, xy, elems, bed, cell=(cell, cell))
