// tsr_host.cpp -- host-side set-up of the two-scale problem: mesh readers and
// CVFE geometry, the effective-conductivity table, solver defaults and the
// phi_1 Pade evaluation.  These run once per run (or on m x m Krylov data)
// and stay on the host; the kernels consume the arrays they produce.
//
// Geometry conventions follow the reference's structure-of-arrays layout
// (include/macro_mesh.h, include/micro_mesh.h); the computations are this
// project's own vertex-centred median-dual construction:
//   * sub-control volume (SCV) of vertex j = quadrilateral (x_j, mid_j, c,
//     mid_{j-1}) of edge midpoints and the element centroid c; its area is
//     half the cross product of its diagonals (c - x_j) x (mid_j - mid_{j-1}).
//     The reference forms the second diagonal as mid_j - mid_{j+1}
//     (src/macro_mesh_properties.cpp:276-279, src/micro_mesh_properties.cpp:
//     252-255), which for triangles gives one sixth of the element instead of
//     one third; this library uses the median-dual areas (each triangle split
//     into three equal SCVs), so triangle CV_area/SCV_area/element_area are
//     twice the reference's values and sum to the mesh area.
//   * SCV face j runs from mid_j to c; its normal is the face vector rotated
//     by -90 degrees for counter-clockwise elements (sign flipped for
//     clockwise ones), length-weighted, pointing from vertex j's SCV into
//     vertex j+1's.
//   * interpolant coefficients: triangles h = a0 x + a1 y + a2, quadrilaterals
//     h = a0 x + a1 y + a2 xy + a3, from the inverse of the vertex matrix.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tsr_capi.h"
#include "tsr_geom.h"
#include "tsr_internal.h"

namespace tsr {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

template <typename T>
static T* alloc_array(size_t n)
{
    T* p = new (std::nothrow) T[n > 0 ? n : 1];
    if (p) std::memset(p, 0, sizeof(T) * (n > 0 ? n : 1));
    return p;
}

// Boundary condition types of the element edges (component-major, edge p
// of element k at p*Ne+k) and which edges are on the boundary: tags -1..-5
// mark nodes; an element edge whose two end nodes carry the same tag gets
// that tag's BC type (later tags win), as the reference does
// (src/macro_mesh_properties.cpp:76-104, 170-190).  Returns 1 if a
// boundary edge names a node out of range.
int macro_bc_edges(int nv, int Mn, int Ne, const int* elements, int n_bedges, const int* bedges,
                   const int* macro_bc, int* bc_edges, unsigned char* is_bedge)
{
    std::vector<unsigned char> flag(5 * (size_t)Mn, 0);
    for (int e = 0; e < n_bedges; ++e) {
        int a = bedges[3 * e], b = bedges[3 * e + 1], tag = bedges[3 * e + 2];
        if (a < 0 || a >= Mn || b < 0 || b >= Mn) return 1;
        if (tag <= -1 && tag >= -5) {
            int j = -tag - 1;
            flag[(size_t)j * Mn + a] = 1;
            flag[(size_t)j * Mn + b] = 1;
        }
    }
    for (int k = 0; k < Ne; ++k)
        for (int j = 0; j < 5; ++j)
            for (int p = 0; p < nv; ++p) {
                int a = elements[(size_t)p * Ne + k];
                int b = elements[(size_t)((p + 1) % nv) * Ne + k];
                if (flag[(size_t)j * Mn + a] && flag[(size_t)j * Mn + b]) {
                    bc_edges[(size_t)p * Ne + k] = macro_bc[j];
                    is_bedge[(size_t)p * Ne + k] = 1;
                }
            }
    return 0;
}

}  // namespace tsr

using namespace tsr;

extern "C" int tsr_version(void) { return 100; }

extern "C" const char* tsr_last_error_message(void) { return tsr::last_error(); }

extern "C" void tsr_macro_mesh_free(macro_mesh_struct* m)
{
    if (!m) return;
    delete[] m->elements;
    delete[] m->nodes;
    delete[] m->shape_funcs;
    delete[] m->normals;
    delete[] m->boundary_edge_midpts;
    delete[] m->boundary_edge_normals;
    delete[] m->boundary_edge_lens;
    delete[] m->boundary_condition_edges;
    delete[] m->CV_area;
    delete[] m->SCV_area;
    delete[] m->midx;
    delete[] m->midy;
    delete[] m->centroid_elements;
    std::memset(m, 0, sizeof *m);
}

extern "C" void tsr_micro_mesh_free(micro_mesh_struct* m)
{
    if (!m) return;
    delete[] m->elements;
    delete[] m->boundary_nodes;
    delete[] m->nodes;
    delete[] m->shape_funcs;
    delete[] m->normals;
    delete[] m->boundary_edges;
    delete[] m->boundary_edge_midpts;
    delete[] m->boundary_edge_normals;
    delete[] m->boundary_edge_lens;
    delete[] m->centroid_elements;
    delete[] m->CV_area;
    delete[] m->midx;
    delete[] m->midy;
    delete[] m->vectors;
    delete[] m->element_area;
    std::memset(m, 0, sizeof *m);
}

extern "C" void tsr_keff_free(Keff_struct* k)
{
    if (!k) return;
    delete[] k->logh_values;
    delete[] k->Keff_values;
    std::memset(k, 0, sizeof *k);
}

static bool valid_elements(int nv, int n_nodes, int n_elems, const int* elems)
{
    if (nv != 3 && nv != 4) return false;
    for (long i = 0; i < (long)n_elems * nv; ++i)
        if (elems[i] < 0 || elems[i] >= n_nodes) return false;
    return true;
}

extern "C" int tsr_macro_mesh_build(int nv, int n_nodes, const double* xy, int n_elems,
                                    const int* elems, int n_bedges, const int* bedges,
                                    const int* macro_bc, macro_mesh_struct* out)
{
    if (!out || !xy || !elems || n_nodes <= 0 || n_elems <= 0 ||
        !valid_elements(nv, n_nodes, n_elems, elems) || (n_bedges > 0 && !bedges) || !macro_bc) {
        set_error("tsr_macro_mesh_build: invalid arguments");
        return TSR_ERR_ARG;
    }
    const int Ne = n_elems, Mn = n_nodes;
    std::memset(out, 0, sizeof *out);
    macro_mesh_struct& m = *out;
    m.no_verts = nv;
    m.no_nodes = Mn;
    m.no_elements = Ne;
    m.elements = alloc_array<int>((size_t)nv * Ne);
    m.nodes = alloc_array<double>(2 * (size_t)Mn);
    m.shape_funcs = alloc_array<double>((size_t)nv * nv * Ne);
    m.normals = alloc_array<double>(2 * (size_t)nv * Ne);
    m.boundary_edge_midpts = alloc_array<double>(4 * (size_t)nv * Ne);
    m.boundary_edge_normals = alloc_array<double>(4 * (size_t)nv * Ne);
    m.boundary_edge_lens = alloc_array<double>(2 * (size_t)nv * Ne);
    m.boundary_condition_edges = alloc_array<int>((size_t)nv * Ne);
    m.CV_area = alloc_array<double>((size_t)Mn);
    m.SCV_area = alloc_array<double>((size_t)nv * Ne);
    m.midx = alloc_array<double>((size_t)nv * Ne);
    m.midy = alloc_array<double>((size_t)nv * Ne);
    m.centroid_elements = alloc_array<double>(2 * (size_t)Ne);
    if (!m.centroid_elements || !m.midy || !m.elements || !m.shape_funcs) {
        tsr_macro_mesh_free(out);
        set_error("tsr_macro_mesh_build: out of host memory");
        return TSR_ERR_ALLOC;
    }
    std::memcpy(m.nodes, xy, sizeof(double) * 2 * (size_t)Mn);
    for (int k = 0; k < Ne; ++k)
        for (int v = 0; v < nv; ++v) m.elements[(size_t)v * Ne + k] = elems[(size_t)k * nv + v];

    std::vector<unsigned char> is_bedge((size_t)nv * Ne, 0);
    if (macro_bc_edges(nv, Mn, Ne, m.elements, n_bedges, bedges, macro_bc, m.boundary_condition_edges,
                       is_bedge.data())) {
        tsr_macro_mesh_free(out);
        set_error("tsr_macro_mesh_build: boundary edge node out of range");
        return TSR_ERR_BOUNDS;
    }

    for (int k = 0; k < Ne; ++k) {
        double xv[4], yv[4];
        for (int j = 0; j < nv; ++j) {
            int v = m.elements[(size_t)j * Ne + k];
            xv[j] = xy[v];
            yv[j] = xy[Mn + v];
        }
        ElemGeom g;
        if (!element_geometry(nv, xv, yv, g)) {
            tsr_macro_mesh_free(out);
            set_error("tsr_macro_mesh_build: degenerate element");
            return TSR_ERR_ARG;
        }
        m.centroid_elements[k] = g.cx;
        m.centroid_elements[Ne + k] = g.cy;
        for (int j = 0; j < nv; ++j) {
            m.SCV_area[(size_t)j * Ne + k] = g.scv[j];
            m.CV_area[m.elements[(size_t)j * Ne + k]] += g.scv[j];
            m.normals[(size_t)(2 * j) * Ne + k] = g.nrm[j][0];
            m.normals[(size_t)(2 * j + 1) * Ne + k] = g.nrm[j][1];
            m.midx[(size_t)j * Ne + k] = g.mid[j][0];
            m.midy[(size_t)j * Ne + k] = g.mid[j][1];
            if (is_bedge[(size_t)j * Ne + k]) {
                for (int s = 0; s < 2; ++s) {
                    m.boundary_edge_lens[(size_t)(2 * j + s) * Ne + k] = g.blen[j][s];
                    for (int d = 0; d < 2; ++d) {
                        m.boundary_edge_midpts[(size_t)(4 * j + 2 * s + d) * Ne + k] = g.bmid[j][s][d];
                        m.boundary_edge_normals[(size_t)(4 * j + 2 * s + d) * Ne + k] = g.bnrm[j][s][d];
                    }
                }
            }
        }
        for (int r = 0; r < nv * nv; ++r) m.shape_funcs[(size_t)r * Ne + k] = g.sf[r];
    }
    return TSR_OK;
}

extern "C" int tsr_micro_mesh_build(double cell_width, double cell_height, int nv,
                                    int n_nodes, const double* xy, int n_elems,
                                    const int* elems, int n_bedges, const int* bedges,
                                    micro_mesh_struct* out)
{
    if (!out || !xy || !elems || n_nodes <= 0 || n_elems <= 0 ||
        !valid_elements(nv, n_nodes, n_elems, elems) || (n_bedges > 0 && !bedges)) {
        set_error("tsr_micro_mesh_build: invalid arguments");
        return TSR_ERR_ARG;
    }
    const int Ne = n_elems, mn = n_nodes;
    std::memset(out, 0, sizeof *out);
    micro_mesh_struct& m = *out;
    m.no_verts = nv;
    m.no_nodes = mn;
    m.no_elements = Ne;
    m.elements = alloc_array<int>((size_t)nv * Ne);
    m.boundary_nodes = alloc_array<int>((size_t)mn);
    m.nodes = alloc_array<double>(2 * (size_t)mn);
    m.shape_funcs = alloc_array<double>((size_t)nv * nv * Ne);
    m.normals = alloc_array<double>(2 * (size_t)nv * Ne);
    m.boundary_edges = alloc_array<int>((size_t)nv * Ne);
    m.boundary_edge_midpts = alloc_array<double>(4 * (size_t)nv * Ne);
    m.boundary_edge_normals = alloc_array<double>(4 * (size_t)nv * Ne);
    m.boundary_edge_lens = alloc_array<double>(2 * (size_t)nv * Ne);
    m.centroid_elements = alloc_array<double>(2 * (size_t)Ne);
    m.CV_area = alloc_array<double>((size_t)mn);
    m.midx = alloc_array<double>((size_t)nv * Ne);
    m.midy = alloc_array<double>((size_t)nv * Ne);
    m.vectors = alloc_array<double>(2 * (size_t)mn);
    m.element_area = alloc_array<double>((size_t)Ne);
    if (!m.element_area || !m.vectors || !m.elements) {
        tsr_micro_mesh_free(out);
        set_error("tsr_micro_mesh_build: out of host memory");
        return TSR_ERR_ALLOC;
    }
    m.cell_area = cell_width * cell_height;
    std::memcpy(m.nodes, xy, sizeof(double) * 2 * (size_t)mn);
    for (int k = 0; k < Ne; ++k)
        for (int v = 0; v < nv; ++v) m.elements[(size_t)v * Ne + k] = elems[(size_t)k * nv + v];
    // tag -1 marks the inclusion boundary (src/micro_mesh_properties.cpp:93-106)
    for (int e = 0; e < n_bedges; ++e) {
        int a = bedges[3 * e], b = bedges[3 * e + 1], tag = bedges[3 * e + 2];
        if (a < 0 || a >= mn || b < 0 || b >= mn) {
            tsr_micro_mesh_free(out);
            set_error("tsr_micro_mesh_build: boundary edge node out of range");
            return TSR_ERR_BOUNDS;
        }
        if (tag == -1) {
            m.boundary_nodes[a] = 1;
            m.boundary_nodes[b] = 1;
        }
    }
    const double cxc = 0.5 * cell_width, cyc = 0.5 * cell_height;
    for (int i = 0; i < mn; ++i) {
        m.vectors[i] = xy[i] - cxc;
        m.vectors[mn + i] = xy[mn + i] - cyc;
    }
    for (int k = 0; k < Ne; ++k) {
        double xv[4], yv[4];
        for (int j = 0; j < nv; ++j) {
            int v = m.elements[(size_t)j * Ne + k];
            xv[j] = xy[v];
            yv[j] = xy[mn + v];
        }
        for (int j = 0; j < nv; ++j) {
            int a = m.elements[(size_t)j * Ne + k];
            int b = m.elements[(size_t)((j + 1) % nv) * Ne + k];
            if (m.boundary_nodes[a] == 1 && m.boundary_nodes[b] == 1)
                m.boundary_edges[(size_t)j * Ne + k] = 1;
        }
        ElemGeom g;
        if (!element_geometry(nv, xv, yv, g)) {
            tsr_micro_mesh_free(out);
            set_error("tsr_micro_mesh_build: degenerate element");
            return TSR_ERR_ARG;
        }
        m.centroid_elements[k] = g.cx;
        m.centroid_elements[Ne + k] = g.cy;
        for (int j = 0; j < nv; ++j) {
            m.CV_area[m.elements[(size_t)j * Ne + k]] += g.scv[j];
            m.element_area[k] += g.scv[j];
            m.normals[(size_t)(2 * j) * Ne + k] = g.nrm[j][0];
            m.normals[(size_t)(2 * j + 1) * Ne + k] = g.nrm[j][1];
            m.midx[(size_t)j * Ne + k] = g.mid[j][0];
            m.midy[(size_t)j * Ne + k] = g.mid[j][1];
            if (m.boundary_edges[(size_t)j * Ne + k]) {
                for (int s = 0; s < 2; ++s) {
                    m.boundary_edge_lens[(size_t)(2 * j + s) * Ne + k] = g.blen[j][s];
                    for (int d = 0; d < 2; ++d) {
                        m.boundary_edge_midpts[(size_t)(4 * j + 2 * s + d) * Ne + k] = g.bmid[j][s][d];
                        m.boundary_edge_normals[(size_t)(4 * j + 2 * s + d) * Ne + k] = g.bnrm[j][s][d];
                    }
                }
            }
        }
        for (int r = 0; r < nv * nv; ++r) m.shape_funcs[(size_t)r * Ne + k] = g.sf[r];
    }
    return TSR_OK;
}

// ---- text readers (formats of tests/Richards_Equation/*.msh) -------------

namespace {
struct Reader {
    FILE* f = nullptr;
    bool ok = true;
    ~Reader() { if (f) std::fclose(f); }
    double real()
    {
        long double v = 0;
        if (std::fscanf(f, "%Lf", &v) != 1) ok = false;
        return (double)v;
    }
    int integer()
    {
        int v = 0;
        if (std::fscanf(f, "%d", &v) != 1) ok = false;
        return v;
    }
};

struct MeshText {
    double w = 0, h = 0;
    int nv = 0, nn = 0, ne = 0, nb = 0;
    std::vector<double> xy;
    std::vector<int> bedges, elems;
};

bool read_mesh_text(const char* file, bool micro, MeshText& mt)
{
    Reader r;
    r.f = std::fopen(file, "r");
    if (!r.f) return false;
    if (micro) {
        mt.w = r.real();
        mt.h = r.real();
    }
    mt.nv = r.integer();
    mt.nn = r.integer();
    if (!r.ok || mt.nn <= 0 || (mt.nv != 3 && mt.nv != 4)) return false;
    mt.xy.assign(2 * (size_t)mt.nn, 0.0);
    for (int i = 0; i < mt.nn; ++i) {
        mt.xy[i] = r.real();
        mt.xy[mt.nn + i] = r.real();
    }
    mt.nb = r.integer();
    if (!r.ok || mt.nb < 0) return false;
    mt.bedges.assign(3 * (size_t)mt.nb, 0);
    for (int e = 0; e < mt.nb; ++e) {
        mt.bedges[3 * e] = r.integer() - 1;
        mt.bedges[3 * e + 1] = r.integer() - 1;
        mt.bedges[3 * e + 2] = r.integer();
    }
    mt.ne = r.integer();
    if (!r.ok || mt.ne <= 0) return false;
    mt.elems.assign((size_t)mt.nv * mt.ne, 0);
    for (int k = 0; k < mt.ne; ++k)
        for (int v = 0; v < mt.nv; ++v) mt.elems[(size_t)k * mt.nv + v] = r.integer() - 1;
    return r.ok;
}
}  // namespace

extern "C" int tsr_macro_mesh_properties(const char* mesh_file, macro_mesh_struct* mesh,
                                         const int* macro_bc)
{
    MeshText mt;
    if (!mesh_file || !read_mesh_text(mesh_file, false, mt)) {
        set_error(std::string("cannot read macro mesh file ") + (mesh_file ? mesh_file : "(null)"));
        return TSR_ERR_IO;
    }
    return tsr_macro_mesh_build(mt.nv, mt.nn, mt.xy.data(), mt.ne, mt.elems.data(), mt.nb,
                                mt.bedges.data(), macro_bc, mesh);
}

extern "C" int tsr_micro_mesh_properties(const char* mesh_file, micro_mesh_struct* mesh)
{
    MeshText mt;
    if (!mesh_file || !read_mesh_text(mesh_file, true, mt)) {
        set_error(std::string("cannot read micro mesh file ") + (mesh_file ? mesh_file : "(null)"));
        return TSR_ERR_IO;
    }
    return tsr_micro_mesh_build(mt.w, mt.h, mt.nv, mt.nn, mt.xy.data(), mt.ne, mt.elems.data(),
                                mt.nb, mt.bedges.data(), mesh);
}

extern "C" int tsr_read_effective_conductivity(const char* file, Keff_struct* keff)
{
    Reader r;
    r.f = file ? std::fopen(file, "r") : nullptr;
    if (!r.f || !keff) {
        set_error(std::string("cannot read Keff file ") + (file ? file : "(null)"));
        return TSR_ERR_IO;
    }
    std::memset(keff, 0, sizeof *keff);
    keff->epsilonA = r.real();
    int n = r.integer();
    keff->logr = r.real();
    keff->logh_first = r.real();
    if (!r.ok || n < 1) {
        set_error("malformed Keff header");
        return TSR_ERR_IO;
    }
    keff->no_hvalues = n;
    keff->logh_values = alloc_array<double>((size_t)n);
    keff->Keff_values = alloc_array<double>(4 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        keff->logh_values[i] = r.real();
        for (int c = 0; c < 4; ++c) keff->Keff_values[(size_t)c * n + i] = r.real();
    }
    if (!r.ok) {
        tsr_keff_free(keff);
        set_error("malformed Keff table");
        return TSR_ERR_IO;
    }
    return TSR_OK;
}

extern "C" int tsr_set_exprem_options(exprem_options_struct* o)
{
    // defaults of src/set_exprem_options.cpp:16-26
    if (!o) return TSR_ERR_ARG;
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
    return TSR_OK;
}

// ---- phi_1 by the (6,6) Pade approximant --------------------------------
//
// phi_1(A) = (e^A - I) A^{-1} ~ D(A)^{-1} N(A) with N = I + sum_i a_i A^{i+1},
// D = I + sum_i b_i A^{i+1}; the coefficients are those of the (6,6) Pade
// approximant of phi_1 given by Hochbruck, Lubich & Selhofer, SIAM J. Sci.
// Comput. 19(5) (1998), p. 1567 (also used by src/phipade.cpp:65-77).  A is
// first scaled by 2^-s with s = max(ceil(1 + log2 ||A||_inf), 0), then
// phi_1(2B) = (e^B + I) phi_1(B) / 2 with e^B = B phi_1(B) + I undoes it.
// Products are plain column-major loops with one fused multiply-add per
// term in ascending k; the same order is used by every evaluation in this
// project so host results are reproducible across builds.

namespace tsr {

// C = A B: element (i, j) is the chain c = fma(A(i, k), B(k, j), c), k
// ascending.  Eight (then four, then one) elements of a column are formed
// side by side, each by its own chain in that order, so the FMA latency is
// hidden without changing a single rounding.
static void matmul(int m, const double* A, const double* B, double* C)
{
    for (int j = 0; j < m; ++j) {
        const double* b = B + (size_t)j * m;
        double* c = C + (size_t)j * m;
        int i = 0;
        for (; i + 8 <= m; i += 8) {
            double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0, c4 = 0.0, c5 = 0.0, c6 = 0.0, c7 = 0.0;
            for (int k = 0; k < m; ++k) {
                const double bk = b[k];
                const double* a = A + (size_t)k * m + i;
                c0 = std::fma(a[0], bk, c0);
                c1 = std::fma(a[1], bk, c1);
                c2 = std::fma(a[2], bk, c2);
                c3 = std::fma(a[3], bk, c3);
                c4 = std::fma(a[4], bk, c4);
                c5 = std::fma(a[5], bk, c5);
                c6 = std::fma(a[6], bk, c6);
                c7 = std::fma(a[7], bk, c7);
            }
            c[i] = c0; c[i + 1] = c1; c[i + 2] = c2; c[i + 3] = c3;
            c[i + 4] = c4; c[i + 5] = c5; c[i + 6] = c6; c[i + 7] = c7;
        }
        for (; i + 4 <= m; i += 4) {
            double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
            for (int k = 0; k < m; ++k) {
                const double bk = b[k];
                const double* a = A + (size_t)k * m + i;
                c0 = std::fma(a[0], bk, c0);
                c1 = std::fma(a[1], bk, c1);
                c2 = std::fma(a[2], bk, c2);
                c3 = std::fma(a[3], bk, c3);
            }
            c[i] = c0; c[i + 1] = c1; c[i + 2] = c2; c[i + 3] = c3;
        }
        for (; i < m; ++i) {
            double cc = 0.0;
            for (int k = 0; k < m; ++k) cc = std::fma(A[(size_t)k * m + i], b[k], cc);
            c[i] = cc;
        }
    }
}

int phipade_host(double* phiH, const double* H, double alpha, int m, int ldH, int ldP)
{
    if (m < 1) return TSR_ERR_ARG;
    if (m == 1) {
        double A = alpha * H[0];
        double eA = std::exp(A);
        if (eA == 1.0) {
            phiH[0] = 1.0;                   // limit phi_1(A) -> 1 as A -> 0 (the reference returns 0 here)
        } else if (eA == 0.0) {
            phiH[0] = -1.0 / A;
        } else {
            phiH[0] = ((eA - 1.0) * A / std::log(eA)) / A;
        }
        return TSR_OK;
    }
    static const double a[6] = {1.0 / 26.0, 5.0 / 156.0, 1.0 / 858.0,
                                1.0 / 5720.0, 1.0 / 205920.0, 1.0 / 8648640.0};
    static const double b[6] = {-6.0 / 13.0, 5.0 / 52.0, -5.0 / 429.0,
                                1.0 / 1144.0, -1.0 / 25740.0, 1.0 / 1235520.0};
    const int mm = m * m;
    // work matrices, kept per thread between calls
    thread_local std::vector<double> work;
    if (work.size() < (size_t)6 * mm) work.resize((size_t)6 * mm);
    double* A = work.data();
    double* P = A + mm;
    double* D = P + mm;
    double* F = D + mm;
    double* E = F + mm;
    double* T = E + mm;
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) A[j * m + i] = alpha * H[j * ldH + i];
    double nrm = 0.0;
    for (int i = 0; i < m; ++i) {
        double s = 0.0;
        for (int j = 0; j < m; ++j) s += std::fabs(A[j * m + i]);
        if (s > nrm || s != s) nrm = s;
    }
    int scale = 0;
    if (nrm > 0.0) {
        double sc = std::ceil(1.0 + std::log(nrm) / std::log(2.0));
        scale = sc > 0.0 ? (int)sc : 0;
    }
    if (scale > 0) {
        double f = 1.0 / std::pow(2.0, (double)scale);
        for (int i = 0; i < mm; ++i) A[i] *= f;
    }
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) {
            double d = (i == j) ? 1.0 : 0.0;
            F[j * m + i] = d;
            D[j * m + i] = d;
            E[j * m + i] = d;
        }
    std::copy(A, A + mm, P);
    for (int i = 0; i < mm; ++i) {
        F[i] = std::fma(a[0], P[i], F[i]);
        D[i] = std::fma(b[0], P[i], D[i]);
    }
    for (int p = 1; p < 6; ++p) {
        matmul(m, P, A, T);
        std::swap(P, T);
        for (int i = 0; i < mm; ++i) {
            F[i] = std::fma(a[p], P[i], F[i]);
            D[i] = std::fma(b[p], P[i], D[i]);
        }
    }
    // F <- D^{-1} F by LU with partial pivoting
    std::vector<int> piv(m);
    for (int k = 0; k < m; ++k) {
        int p = k;
        double best = std::fabs(D[k * m + k]);
        for (int i = k + 1; i < m; ++i)
            if (std::fabs(D[k * m + i]) > best) { best = std::fabs(D[k * m + i]); p = i; }
        if (!(best > 0.0)) return TSR_ERR_SINGULAR;
        piv[k] = p;
        if (p != k) {
            for (int j = 0; j < m; ++j) std::swap(D[j * m + k], D[j * m + p]);
            for (int j = 0; j < m; ++j) std::swap(F[j * m + k], F[j * m + p]);
        }
        double inv = 1.0 / D[k * m + k];
        for (int i = k + 1; i < m; ++i) {
            double l = D[k * m + i] * inv;
            D[k * m + i] = l;
            for (int j = k + 1; j < m; ++j) D[j * m + i] = std::fma(-l, D[j * m + k], D[j * m + i]);
            for (int j = 0; j < m; ++j) F[j * m + i] = std::fma(-l, F[j * m + k], F[j * m + i]);
        }
    }
    for (int j = 0; j < m; ++j)
        for (int i = m - 1; i >= 0; --i) {
            double s = F[j * m + i];
            for (int k = i + 1; k < m; ++k) s = std::fma(-D[k * m + i], F[j * m + k], s);
            F[j * m + i] = s / D[i * m + i];
        }
    if (scale > 0) {
        matmul(m, A, F, T);                                // E = A phi + I
        for (int i = 0; i < mm; ++i) E[i] += T[i];
        for (int it = 0; it < scale; ++it) {
            if (it > 0) {
                matmul(m, E, E, T);                        // E = E^2
                std::swap(E, T);
            }
            matmul(m, E, F, T);                            // phi = (E phi + phi) / 2
            for (int i = 0; i < mm; ++i) F[i] = 0.5 * (T[i] + F[i]);
        }
    }
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) phiH[j * ldP + i] = F[j * m + i];
    return TSR_OK;
}

}  // namespace tsr

extern "C" int tsr_phipade(double* phiH, const double* H, double alpha, int m, int MaxKrylov)
{
    if (!phiH || !H || m < 1 || m > MaxKrylov) {
        set_error("tsr_phipade: invalid arguments");
        return TSR_ERR_ARG;
    }
    int rc = tsr::phipade_host(phiH, H, alpha, m, MaxKrylov + 1, MaxKrylov);
    if (rc == TSR_ERR_SINGULAR) set_error("phipade: singular Pade denominator");
    return rc;
}

// ---- solution calibration --------------------------------------------------
// The micro boundary unknowns are not evolved (G is 0 there; the cell sees
// the macro interpolant instead), so, as src/save_solution.cpp:256-318 does
// before writing, their stored values are overwritten with the macro
// interpolant at centroid_k + s vectors_l (model_type 1: the centroid).

extern "C" int tsr_save_solution(const char* solution_file, const double* tspan, double* tspan_solns,
                                 int no_solns, const user_data_struct* ud)
{
    if (!solution_file || !tspan || !tspan_solns || no_solns < 0) return TSR_ERR_ARG;
    long long N = 0;
    if (ud) {
        N = (long long)ud->macro_mesh.no_nodes + (long long)ud->macro_mesh.no_elements * ud->micro_mesh.no_nodes;
        // the reference calibrates the stored rows in place before writing
        for (int j = 0; j <= no_solns; ++j) {
            int rc = tsr_calibrate_micro_boundary(ud, nullptr, tspan_solns + (size_t)j * (size_t)N);
            if (rc) return rc;
        }
    } else {
        return TSR_ERR_ARG;
    }
    FILE* f = std::fopen(solution_file, "w");
    if (!f) {
        set_error(std::string("cannot open ") + solution_file);
        return TSR_ERR_IO;
    }
    // the reference's layout: the row count, then per row the time and the
    // N values, scientific with 20 digits after the point
    bool ok = std::fprintf(f, "%d\n", no_solns + 1) > 0;
    for (int j = 0; j <= no_solns && ok; ++j) {
        ok = std::fprintf(f, "%.20e", j == 0 ? 0.0 : tspan[j]) > 0;
        const double* row = tspan_solns + (size_t)j * (size_t)N;
        for (long long k = 0; k < N && ok; ++k) ok = std::fprintf(f, " %.20e", row[k]) > 0;
        ok = ok && std::fputc('\n', f) != EOF;
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) {
        set_error(std::string("write failed: ") + solution_file);
        return TSR_ERR_IO;
    }
    return TSR_OK;
}

extern "C" int tsr_calibrate_micro_boundary(const user_data_struct* ud, const tsr_model_ext* ext,
                                            double* u)
{
    if (!ud || !u) return TSR_ERR_ARG;
    const macro_mesh_struct& M = ud->macro_mesh;
    const micro_mesh_struct& m = ud->micro_mesh;
    const int nv = M.no_verts, Ne = M.no_elements, Mn = M.no_nodes, mn = m.no_nodes;
    const double* scale = ext ? ext->cell_scale : nullptr;
    for (int k = 0; k < Ne; ++k) {
        double al[4];
        for (int q = 0; q < nv; ++q) {
            double a = M.shape_funcs[(size_t)(q * nv) * Ne + k] * u[M.elements[k]];
            for (int i = 1; i < nv; ++i)
                a = std::fma(M.shape_funcs[(size_t)(q * nv + i) * Ne + k],
                             u[M.elements[(size_t)i * Ne + k]], a);
            al[q] = a;
        }
        const double s = scale ? scale[k] : 1.0;
        const double cx = M.centroid_elements[k], cy = M.centroid_elements[Ne + k];
        for (int l = 0; l < mn; ++l) {
            if (m.boundary_nodes[l] != 1) continue;
            double px = cx, py = cy;
            if (ud->model_type != 1) {
                px = std::fma(s, m.vectors[l], cx);
                py = std::fma(s, m.vectors[mn + l], cy);
            }
            double v = (nv == 3) ? std::fma(al[0], px, std::fma(al[1], py, al[2]))
                                 : std::fma(al[0], px, std::fma(al[1], py, std::fma(al[2], px * py, al[3])));
            u[(size_t)Mn + (size_t)k * mn + l] = v;
        }
    }
    return TSR_OK;
}
