// tsr_geom.h -- the CVFE geometry of one mesh element (centroid, sub-control
// volumes, SCV face normals and midpoints, boundary half-edges, interpolant
// coefficients), shared by the host mesh builders (tsr_host.cpp) and the
// device macro-mesh builder (tsr_meshdev.cu): one source, so both compute
// the same operations in the same order and give the same bits (host code
// without contraction, device code with -fmad=false; sqrt and division
// correctly rounded on both).
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define TSR_HD __host__ __device__
#else
#define TSR_HD
#endif

namespace tsr {

TSR_HD inline int orientation_sign(const double* xv, const double* yv, int nv)
{
    // sum (x_{j+1} - x_j)(y_{j+1} + y_j) is positive for clockwise vertices
    double s = 0.0;
    for (int j = 0; j < nv; ++j) {
        int jn = (j + 1) % nv;
        s += (xv[jn] - xv[j]) * (yv[jn] + yv[j]);
    }
    return (s < 0.0) ? 1 : ((s > 0.0) ? -1 : 0);  // +1 for counter-clockwise
}

// Inverse of the n x n matrix M (row major) by Gauss-Jordan elimination with
// partial pivoting; returns false if singular.
TSR_HD inline bool invert_small(int n, const double* M, double* Minv)
{
    double a[4][8];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 2 * n; ++j)
            a[i][j] = (j < n) ? M[i * n + j] : ((j - n == i) ? 1.0 : 0.0);
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(a[r][c]) > fabs(a[p][c])) p = r;
        if (a[p][c] == 0.0) return false;
        if (p != c)
            for (int j = 0; j < 2 * n; ++j) {
                const double t = a[p][j];
                a[p][j] = a[c][j];
                a[c][j] = t;
            }
        double inv = 1.0 / a[c][c];
        for (int j = 0; j < 2 * n; ++j) a[c][j] *= inv;
        for (int r = 0; r < n; ++r) {
            if (r == c || a[r][c] == 0.0) continue;
            double f = a[r][c];
            for (int j = 0; j < 2 * n; ++j) a[r][j] -= f * a[c][j];
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) Minv[i * n + j] = a[i][n + j];
    return true;
}

// Element geometry shared by the macro and micro builders.
struct ElemGeom {
    int nv;
    double cx, cy;
    double scv[4];
    double nrm[4][2];
    double mid[4][2];        // SCV face midpoints
    double sf[16];           // coefficient m of vertex i at m*nv+i
    double blen[4][2];
    double bmid[4][2][2];
    double bnrm[4][2][2];
};

TSR_HD inline bool element_geometry(int nv, const double* xv, const double* yv, ElemGeom& g)
{
    g.nv = nv;
    g.cx = 0.0;
    g.cy = 0.0;
    for (int j = 0; j < nv; ++j) { g.cx += xv[j]; g.cy += yv[j]; }
    g.cx /= (double)nv;
    g.cy /= (double)nv;
    int sgn = orientation_sign(xv, yv, nv);
    double em[4][2];
    for (int j = 0; j < nv; ++j) {
        int jn = (j + 1) % nv;
        em[j][0] = 0.5 * (xv[j] + xv[jn]);
        em[j][1] = 0.5 * (yv[j] + yv[jn]);
    }
    for (int j = 0; j < nv; ++j) {
        int jp = (j + nv - 1) % nv;
        double d1x = g.cx - xv[j], d1y = g.cy - yv[j];
        double d2x = em[j][0] - em[jp][0], d2y = em[j][1] - em[jp][1];
        g.scv[j] = 0.5 * fabs(d1x * d2y - d1y * d2x);
        double fx = g.cx - em[j][0], fy = g.cy - em[j][1];
        g.nrm[j][0] = sgn * fy;
        g.nrm[j][1] = -sgn * fx;
        g.mid[j][0] = 0.5 * (em[j][0] + g.cx);
        g.mid[j][1] = 0.5 * (em[j][1] + g.cy);
        int jn = (j + 1) % nv;
        double tx0 = em[j][0] - xv[j], ty0 = em[j][1] - yv[j];
        double tx1 = xv[jn] - em[j][0], ty1 = yv[jn] - em[j][1];
        g.blen[j][0] = sqrt(tx0 * tx0 + ty0 * ty0);
        g.blen[j][1] = sqrt(tx1 * tx1 + ty1 * ty1);
        g.bmid[j][0][0] = 0.5 * (xv[j] + em[j][0]);
        g.bmid[j][0][1] = 0.5 * (yv[j] + em[j][1]);
        g.bmid[j][1][0] = 0.5 * (xv[jn] + em[j][0]);
        g.bmid[j][1][1] = 0.5 * (yv[jn] + em[j][1]);
        g.bnrm[j][0][0] = sgn * ty0;
        g.bnrm[j][0][1] = -sgn * tx0;
        g.bnrm[j][1][0] = sgn * ty1;
        g.bnrm[j][1][1] = -sgn * tx1;
    }
    // interpolant: rows of the vertex matrix are (x, y, 1) or (x, y, xy, 1);
    // coefficient m of vertex i is Minv[m][i]
    double M[16], Mi[16];
    for (int i = 0; i < nv; ++i) {
        if (nv == 3) {
            M[i * 3 + 0] = xv[i];
            M[i * 3 + 1] = yv[i];
            M[i * 3 + 2] = 1.0;
        } else {
            M[i * 4 + 0] = xv[i];
            M[i * 4 + 1] = yv[i];
            M[i * 4 + 2] = xv[i] * yv[i];
            M[i * 4 + 3] = 1.0;
        }
    }
    if (!invert_small(nv, M, Mi)) return false;
    for (int m = 0; m < nv; ++m)
        for (int i = 0; i < nv; ++i) g.sf[m * nv + i] = Mi[m * nv + i];
    return true;
}


}  // namespace tsr
