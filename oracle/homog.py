"""CPU restatement of the unit-cell homogenisation (tsr_keff_homogenize) --
TEST INFRASTRUCTURE ONLY.

The same discrete cell problem, formed independently: face fractions of the
periodic grid from the inclusion's triangles (each face's cross-section
with every triangle, summed), the cut-face finite-volume operator assembled
as a scipy sparse matrix, and a direct solve (one node per connected block
pinned) instead of conjugate gradients.  Small grids only (the tests use
64-128 cells per side).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl


def face_fractions(tri_xy, width, height, Mx, My):
    """fx[j, i]: fraction in A of the x-face at x = (i+1) hx, y in row j;
    fy[j, i]: fraction in A of the y-face at y = (j+1) hy, x in column i."""
    hx, hy = width / Mx, height / My
    fx = np.ones((My, Mx))
    fy = np.ones((My, Mx))
    for t in tri_xy:                                      # t: 3 x 2
        xs, ys = t[:, 0], t[:, 1]
        for i in range(Mx):
            xf = (i + 1) * hx
            if not (xs.min() <= xf <= xs.max()):
                continue
            iv = _section(xf, xs, ys)
            if iv is None:
                continue
            for j in range(My):
                l = min(iv[1], (j + 1) * hy) - max(iv[0], j * hy)
                if l > 0:
                    fx[j, i] -= l / hy
        for j in range(My):
            yf = (j + 1) * hy
            if not (ys.min() <= yf <= ys.max()):
                continue
            iv = _section(yf, ys, xs)
            if iv is None:
                continue
            for i in range(Mx):
                l = min(iv[1], (i + 1) * hx) - max(iv[0], i * hx)
                if l > 0:
                    fy[j, i] -= l / hx
    return np.clip(fx, 0.0, 1.0), np.clip(fy, 0.0, 1.0)


def _section(fixed, c, o):
    """Interval in o of the triangle (c, o) on the line c = fixed."""
    lo, hi, hits = np.inf, -np.inf, 0
    for e in range(3):
        f = (e + 1) % 3
        if (c[e] - fixed) * (c[f] - fixed) > 0:
            continue
        if c[e] == c[f]:
            if c[e] != fixed:
                continue
            lo, hi, hits = min(lo, o[e], o[f]), max(hi, o[e], o[f]), hits + 2
            continue
        v = o[e] + (fixed - c[e]) / (c[f] - c[e]) * (o[f] - o[e])
        lo, hi, hits = min(lo, v), max(hi, v), hits + 1
    return (lo, hi) if hits >= 2 else None


def homogenize(tri_xy, width, height, Mx, My):
    """(Khom 2x2 with K_A = 1, epsA) of the perforated periodic cell."""
    hx, hy = width / Mx, height / My
    fx, fy = face_fractions(tri_xy, width, height, Mx, My)
    wx, wy = fx * hy / hx, fy * hx / hy
    idx = np.arange(Mx * My).reshape(My, Mx)
    east, north = np.roll(idx, -1, axis=1), np.roll(idx, -1, axis=0)
    rows = np.concatenate([idx.ravel(), east.ravel(), idx.ravel(), north.ravel()])
    cols = np.concatenate([east.ravel(), idx.ravel(), north.ravel(), idx.ravel()])
    vals = np.concatenate([-wx.ravel(), -wx.ravel(), -wy.ravel(), -wy.ravel()])
    L = sp.coo_matrix((vals, (rows, cols)), shape=(Mx * My,) * 2).tocsr()
    diag = -np.asarray(L.sum(axis=1)).ravel()
    L = L + sp.diags(diag)
    # pin one unknown per connected block; isolated cells get the identity
    ncomp, lab = sp.csgraph.connected_components(sp.csr_matrix((np.abs(L.data) > 0, L.indices, L.indptr),
                                                               shape=L.shape), directed=False)
    L = L.tolil()
    pinned = set()
    for c in range(ncomp):
        p = int(np.nonzero(lab == c)[0][0])
        pinned.add(p)
        L[p, :] = 0.0
        L[p, p] = 1.0
    L = L.tocsr()
    K = np.zeros((2, 2))
    for d in range(2):
        if d == 0:
            rhs = hy * (fx - np.roll(fx, 1, axis=1))
        else:
            rhs = hx * (fy - np.roll(fy, 1, axis=0))
        rhs = rhs.ravel().copy()
        for p in pinned:
            rhs[p] = 0.0
        chi = spl.spsolve(L, rhs).reshape(My, Mx)
        qx = np.sum((wx * (np.roll(chi, -1, axis=1) - chi) + (fx * hy if d == 0 else 0.0)) * hx)
        qy = np.sum((wy * (np.roll(chi, -1, axis=0) - chi) + (fy * hx if d == 1 else 0.0)) * hy)
        K[0, d], K[1, d] = qx / (width * height), qy / (width * height)
    area_b = sum(0.5 * abs((t[1, 0] - t[0, 0]) * (t[2, 1] - t[0, 1]) - (t[2, 0] - t[0, 0]) * (t[1, 1] - t[0, 1]))
                 for t in tri_xy)
    return K, 1.0 - area_b / (width * height)
