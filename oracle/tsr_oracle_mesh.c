/*
 * tsr_oracle_mesh.c -- CPU restatement of the mesh preprocessing and solver
 * defaults, for the oracle's own problems.  TEST INFRASTRUCTURE ONLY: the
 * CPU arm of the benchmark builds its problems with these functions, so
 * that timing the reference's CPU path loads no part of the GB300 library;
 * a test compares the arrays with the library's (to rounding) and with the
 * reference's own preprocessing (golden vectors).
 *
 * What it restates: macro_mesh_properties / micro_mesh_properties
 * (src/macro_mesh_properties.cpp:241-456, src/micro_mesh_properties.cpp:
 * 216-428) -- per element the centroid, the median-dual sub-control volumes
 * (vertex, edge midpoint, centroid, previous edge midpoint), the SCV faces
 * from each edge midpoint to the centroid with their length-weighted
 * normals and midpoints, the boundary half-edges, and the interpolant
 * coefficients (P1 triangles h = a0 x + a1 y + a2, bilinear quadrilaterals
 * h = a0 x + a1 y + a2 xy + a3); boundary tags -1..-5 of the macro mesh
 * mapped to BC types through macro_bc (src/macro_mesh_properties.cpp:
 * 76-104, 170-190), tag -1 of the micro mesh marking the inclusion boundary
 * (src/micro_mesh_properties.cpp:93-106).  Triangle SCVs are the
 * median-dual thirds (the reference's own code forms one sixth, a recorded
 * quirk).  Layouts: component-major SoA, array[c * count + index].
 * Defaults of the solver: src/set_exprem_options.cpp:16-26.
 *
 * Formulation (independent of the library's): closed-form P1 coefficients
 * from the doubled signed area; an LU solve with partial pivoting for the
 * bilinear rows; shoelace areas of the SCV quadrilaterals.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../include/tsr_types.h"

typedef struct {
    double cx, cy;
    double scv[4];
    double nrm[4][2], mid[4][2];
    double blen[4][2], bmid[4][2][2], bnrm[4][2][2];
    double sf[16];          /* coefficient m of vertex i at m * nv + i */
} og_elem;

static double shoelace(const double* px, const double* py, int n)
{
    double a = 0.0;
    for (int i = 0; i < n; ++i) {
        int j = (i + 1) % n;
        a += px[i] * py[j] - px[j] * py[i];
    }
    return 0.5 * a;
}

/* solve the 4x4 system A X = I (rows (x, y, xy, 1)) by LU with partial
 * pivoting; X column i = coefficients of vertex i's basis function */
static int bilinear_coeffs(const double* xv, const double* yv, double* sf)
{
    double A[4][4], B[4][4];
    for (int i = 0; i < 4; ++i) {
        A[i][0] = xv[i];
        A[i][1] = yv[i];
        A[i][2] = xv[i] * yv[i];
        A[i][3] = 1.0;
        for (int j = 0; j < 4; ++j) B[i][j] = (i == j) ? 1.0 : 0.0;
    }
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (fabs(A[r][c]) > fabs(A[p][c])) p = r;
        if (A[p][c] == 0.0) return 1;
        if (p != c)
            for (int j = 0; j < 4; ++j) {
                double t = A[p][j]; A[p][j] = A[c][j]; A[c][j] = t;
                t = B[p][j]; B[p][j] = B[c][j]; B[c][j] = t;
            }
        for (int r = c + 1; r < 4; ++r) {
            double f = A[r][c] / A[c][c];
            if (f == 0.0) continue;
            for (int j = c; j < 4; ++j) A[r][j] -= f * A[c][j];
            for (int j = 0; j < 4; ++j) B[r][j] -= f * B[c][j];
        }
    }
    /* back substitution, one right-hand side per vertex i */
    for (int i = 0; i < 4; ++i) {
        double x[4];
        for (int r = 3; r >= 0; --r) {
            double s = B[r][i];
            for (int j = r + 1; j < 4; ++j) s -= A[r][j] * x[j];
            x[r] = s / A[r][r];
        }
        for (int m = 0; m < 4; ++m) sf[m * 4 + i] = x[m];
    }
    return 0;
}

static int element(int nv, const double* xv, const double* yv, og_elem* g)
{
    double sx = 0.0, sy = 0.0;
    for (int j = 0; j < nv; ++j) { sx += xv[j]; sy += yv[j]; }
    g->cx = sx / nv;
    g->cy = sy / nv;
    const double area = shoelace(xv, yv, nv);
    if (area == 0.0) return 1;
    const double o = area > 0.0 ? 1.0 : -1.0;        /* +1 counter-clockwise */
    double ex[4], ey[4];
    for (int j = 0; j < nv; ++j) {
        int n = (j + 1) % nv;
        ex[j] = 0.5 * (xv[j] + xv[n]);
        ey[j] = 0.5 * (yv[j] + yv[n]);
    }
    for (int j = 0; j < nv; ++j) {
        int p = (j + nv - 1) % nv, n = (j + 1) % nv;
        double qx[4] = {xv[j], ex[j], g->cx, ex[p]}, qy[4] = {yv[j], ey[j], g->cy, ey[p]};
        g->scv[j] = fabs(shoelace(qx, qy, 4));
        /* face from the edge midpoint to the centroid, normal = face
         * vector turned clockwise (counter-clockwise element) */
        double fx = g->cx - ex[j], fy = g->cy - ey[j];
        g->nrm[j][0] = o * fy;
        g->nrm[j][1] = -o * fx;
        g->mid[j][0] = 0.5 * (ex[j] + g->cx);
        g->mid[j][1] = 0.5 * (ey[j] + g->cy);
        /* boundary half-edges vertex j -> midpoint -> vertex j+1 */
        double t[2][2] = {{ex[j] - xv[j], ey[j] - yv[j]}, {xv[n] - ex[j], yv[n] - ey[j]}};
        double a[2][2] = {{xv[j], yv[j]}, {xv[n], yv[n]}};
        for (int s = 0; s < 2; ++s) {
            g->blen[j][s] = hypot(t[s][0], t[s][1]);
            g->bmid[j][s][0] = 0.5 * (a[s][0] + ex[j]);
            g->bmid[j][s][1] = 0.5 * (a[s][1] + ey[j]);
            g->bnrm[j][s][0] = o * t[s][1];
            g->bnrm[j][s][1] = -o * t[s][0];
        }
    }
    if (nv == 3) {
        /* P1: basis of vertex i = (a x + b y + c) / (2 area) */
        const double d = 2.0 * area;
        for (int i = 0; i < 3; ++i) {
            int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
            g->sf[0 * 3 + i] = (yv[i1] - yv[i2]) / d;
            g->sf[1 * 3 + i] = (xv[i2] - xv[i1]) / d;
            g->sf[2 * 3 + i] = (xv[i1] * yv[i2] - xv[i2] * yv[i1]) / d;
        }
        return 0;
    }
    return bilinear_coeffs(xv, yv, g->sf);
}

static void* zalloc(size_t n, size_t sz) { return calloc(n > 0 ? n : 1, sz); }

void oracle_macro_mesh_free(macro_mesh_struct* m)
{
    if (!m) return;
    free(m->elements); free(m->nodes); free(m->shape_funcs); free(m->normals);
    free(m->boundary_edge_midpts); free(m->boundary_edge_normals); free(m->boundary_edge_lens);
    free(m->boundary_condition_edges); free(m->CV_area); free(m->SCV_area);
    free(m->midx); free(m->midy); free(m->centroid_elements);
    memset(m, 0, sizeof *m);
}

void oracle_micro_mesh_free(micro_mesh_struct* m)
{
    if (!m) return;
    free(m->elements); free(m->boundary_nodes); free(m->nodes); free(m->shape_funcs);
    free(m->normals); free(m->boundary_edges); free(m->boundary_edge_midpts);
    free(m->boundary_edge_normals); free(m->boundary_edge_lens); free(m->centroid_elements);
    free(m->CV_area); free(m->midx); free(m->midy); free(m->vectors); free(m->element_area);
    memset(m, 0, sizeof *m);
}

/* element geometry into the SoA arrays of element k (both mesh kinds) */
static void store(int nv, int Ne, int k, const og_elem* g, const int* is_b, int* elements,
                  double* CV, double* SCV, double* normals, double* midx, double* midy,
                  double* blen, double* bmid, double* bnrm, double* cent, double* sf)
{
    cent[k] = g->cx;
    cent[Ne + k] = g->cy;
    for (int j = 0; j < nv; ++j) {
        if (SCV) SCV[(size_t)j * Ne + k] = g->scv[j];
        CV[elements[(size_t)j * Ne + k]] += g->scv[j];
        normals[(size_t)(2 * j) * Ne + k] = g->nrm[j][0];
        normals[(size_t)(2 * j + 1) * Ne + k] = g->nrm[j][1];
        midx[(size_t)j * Ne + k] = g->mid[j][0];
        midy[(size_t)j * Ne + k] = g->mid[j][1];
        if (!is_b[(size_t)j * Ne + k]) continue;
        for (int s = 0; s < 2; ++s) {
            blen[(size_t)(2 * j + s) * Ne + k] = g->blen[j][s];
            for (int d = 0; d < 2; ++d) {
                bmid[(size_t)(4 * j + 2 * s + d) * Ne + k] = g->bmid[j][s][d];
                bnrm[(size_t)(4 * j + 2 * s + d) * Ne + k] = g->bnrm[j][s][d];
            }
        }
    }
    for (int r = 0; r < nv * nv; ++r) sf[(size_t)r * Ne + k] = g->sf[r];
}

static int check_elems(int nv, int n, int ne, const int* el)
{
    if (nv != 3 && nv != 4) return 1;
    for (long i = 0; i < (long)ne * nv; ++i)
        if (el[i] < 0 || el[i] >= n) return 1;
    return 0;
}

/* Same arguments and output as tsr_macro_mesh_build (0-based element-major
 * elems, boundary edges (a, b, tag)); returns 0 or TSR_ERR_ARG. */
int oracle_macro_mesh_build(int nv, int Mn, const double* xy, int Ne, const int* elems,
                            int n_bedges, const int* bedges, const int* macro_bc,
                            macro_mesh_struct* m)
{
    if (!m || !xy || !elems || Mn <= 0 || Ne <= 0 || check_elems(nv, Mn, Ne, elems) || !macro_bc)
        return 5;
    memset(m, 0, sizeof *m);
    m->no_verts = nv;
    m->no_nodes = Mn;
    m->no_elements = Ne;
    const size_t nvNe = (size_t)nv * Ne;
    m->elements = (int*)zalloc(nvNe, sizeof(int));
    m->nodes = (double*)zalloc(2 * (size_t)Mn, sizeof(double));
    m->shape_funcs = (double*)zalloc(nv * nvNe, sizeof(double));
    m->normals = (double*)zalloc(2 * nvNe, sizeof(double));
    m->boundary_edge_midpts = (double*)zalloc(4 * nvNe, sizeof(double));
    m->boundary_edge_normals = (double*)zalloc(4 * nvNe, sizeof(double));
    m->boundary_edge_lens = (double*)zalloc(2 * nvNe, sizeof(double));
    m->boundary_condition_edges = (int*)zalloc(nvNe, sizeof(int));
    m->CV_area = (double*)zalloc((size_t)Mn, sizeof(double));
    m->SCV_area = (double*)zalloc(nvNe, sizeof(double));
    m->midx = (double*)zalloc(nvNe, sizeof(double));
    m->midy = (double*)zalloc(nvNe, sizeof(double));
    m->centroid_elements = (double*)zalloc(2 * (size_t)Ne, sizeof(double));
    memcpy(m->nodes, xy, sizeof(double) * 2 * (size_t)Mn);
    for (int k = 0; k < Ne; ++k)
        for (int v = 0; v < nv; ++v) m->elements[(size_t)v * Ne + k] = elems[(size_t)k * nv + v];
    unsigned char* tagged = (unsigned char*)zalloc(5 * (size_t)Mn, 1);
    int* is_b = (int*)zalloc(nvNe, sizeof(int));
    for (int e = 0; e < n_bedges; ++e) {
        int a = bedges[3 * e], b = bedges[3 * e + 1], tag = bedges[3 * e + 2];
        if (a < 0 || a >= Mn || b < 0 || b >= Mn) {
            free(tagged); free(is_b); oracle_macro_mesh_free(m);
            return 3;
        }
        if (tag <= -1 && tag >= -5) {
            tagged[(size_t)(-tag - 1) * Mn + a] = 1;
            tagged[(size_t)(-tag - 1) * Mn + b] = 1;
        }
    }
    for (int k = 0; k < Ne; ++k)
        for (int j = 0; j < 5; ++j)            /* later tags win */
            for (int p = 0; p < nv; ++p) {
                int a = m->elements[(size_t)p * Ne + k], b = m->elements[(size_t)((p + 1) % nv) * Ne + k];
                if (tagged[(size_t)j * Mn + a] && tagged[(size_t)j * Mn + b]) {
                    m->boundary_condition_edges[(size_t)p * Ne + k] = macro_bc[j];
                    is_b[(size_t)p * Ne + k] = 1;
                }
            }
    int rc = 0;
    for (int k = 0; k < Ne && !rc; ++k) {
        double xv[4], yv[4];
        for (int j = 0; j < nv; ++j) {
            int v = m->elements[(size_t)j * Ne + k];
            xv[j] = xy[v];
            yv[j] = xy[Mn + v];
        }
        og_elem g;
        if (element(nv, xv, yv, &g)) {
            rc = 5;
            break;
        }
        store(nv, Ne, k, &g, is_b, m->elements, m->CV_area, m->SCV_area, m->normals, m->midx,
              m->midy, m->boundary_edge_lens, m->boundary_edge_midpts, m->boundary_edge_normals,
              m->centroid_elements, m->shape_funcs);
    }
    free(tagged);
    free(is_b);
    if (rc) oracle_macro_mesh_free(m);
    return rc;
}

/* Same arguments and output as tsr_micro_mesh_build. */
int oracle_micro_mesh_build(double cw, double ch, int nv, int mn, const double* xy, int Ne,
                            const int* elems, int n_bedges, const int* bedges, micro_mesh_struct* m)
{
    if (!m || !xy || !elems || mn <= 0 || Ne <= 0 || check_elems(nv, mn, Ne, elems)) return 5;
    memset(m, 0, sizeof *m);
    m->no_verts = nv;
    m->no_nodes = mn;
    m->no_elements = Ne;
    const size_t nvNe = (size_t)nv * Ne;
    m->elements = (int*)zalloc(nvNe, sizeof(int));
    m->boundary_nodes = (int*)zalloc((size_t)mn, sizeof(int));
    m->nodes = (double*)zalloc(2 * (size_t)mn, sizeof(double));
    m->shape_funcs = (double*)zalloc(nv * nvNe, sizeof(double));
    m->normals = (double*)zalloc(2 * nvNe, sizeof(double));
    m->boundary_edges = (int*)zalloc(nvNe, sizeof(int));
    m->boundary_edge_midpts = (double*)zalloc(4 * nvNe, sizeof(double));
    m->boundary_edge_normals = (double*)zalloc(4 * nvNe, sizeof(double));
    m->boundary_edge_lens = (double*)zalloc(2 * nvNe, sizeof(double));
    m->centroid_elements = (double*)zalloc(2 * (size_t)Ne, sizeof(double));
    m->CV_area = (double*)zalloc((size_t)mn, sizeof(double));
    m->midx = (double*)zalloc(nvNe, sizeof(double));
    m->midy = (double*)zalloc(nvNe, sizeof(double));
    m->vectors = (double*)zalloc(2 * (size_t)mn, sizeof(double));
    m->element_area = (double*)zalloc((size_t)Ne, sizeof(double));
    m->cell_area = cw * ch;
    memcpy(m->nodes, xy, sizeof(double) * 2 * (size_t)mn);
    for (int k = 0; k < Ne; ++k)
        for (int v = 0; v < nv; ++v) m->elements[(size_t)v * Ne + k] = elems[(size_t)k * nv + v];
    for (int e = 0; e < n_bedges; ++e) {
        int a = bedges[3 * e], b = bedges[3 * e + 1];
        if (a < 0 || a >= mn || b < 0 || b >= mn) {
            oracle_micro_mesh_free(m);
            return 3;
        }
        if (bedges[3 * e + 2] == -1) m->boundary_nodes[a] = m->boundary_nodes[b] = 1;
    }
    for (int i = 0; i < mn; ++i) {
        m->vectors[i] = xy[i] - 0.5 * cw;
        m->vectors[mn + i] = xy[mn + i] - 0.5 * ch;
    }
    for (int k = 0; k < Ne; ++k)
        for (int j = 0; j < nv; ++j) {
            int a = m->elements[(size_t)j * Ne + k], b = m->elements[(size_t)((j + 1) % nv) * Ne + k];
            if (m->boundary_nodes[a] == 1 && m->boundary_nodes[b] == 1) m->boundary_edges[(size_t)j * Ne + k] = 1;
        }
    for (int k = 0; k < Ne; ++k) {
        double xv[4], yv[4];
        for (int j = 0; j < nv; ++j) {
            int v = m->elements[(size_t)j * Ne + k];
            xv[j] = xy[v];
            yv[j] = xy[mn + v];
        }
        og_elem g;
        if (element(nv, xv, yv, &g)) {
            oracle_micro_mesh_free(m);
            return 5;
        }
        store(nv, Ne, k, &g, m->boundary_edges, m->elements, m->CV_area, NULL, m->normals, m->midx,
              m->midy, m->boundary_edge_lens, m->boundary_edge_midpts, m->boundary_edge_normals,
              m->centroid_elements, m->shape_funcs);
        for (int j = 0; j < nv; ++j) m->element_area[k] += g.scv[j];
    }
    return 0;
}

/* defaults of src/set_exprem_options.cpp:16-26 */
int oracle_set_exprem_options(exprem_options_struct* o)
{
    if (!o) return 5;
    o->AbsTol = 1.0e-5;
    o->RelTol = 1.0e-5;
    o->MinKrylov = 2;
    o->MaxKrylov = 100;
    o->MinStep = 1.0e-10;
    o->MaxStep = 1000.0;
    o->MaxNumSteps = 100000;
    o->SafetyFac = 0.8;
    o->MinStepDecFac = 0.1;
    o->MaxStepIncFac = 1.1;
    o->InitStep = 1.0e-3;
    return 0;
}
