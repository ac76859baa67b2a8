// tsr_meshdev.cu -- the macro mesh's CVFE geometry computed on the GPU, the
// step the reference does on the host once per run
// (src/macro_mesh_properties.cpp:241-456).  tsr_macro_mesh_build_device
// takes the arguments of tsr_macro_mesh_build and fills the same host
// struct: one thread per element evaluates element_geometry (tsr_geom.h,
// the host builder's own code) and one thread per node gathers its
// control-volume area over its elements in ascending element order, the
// order in which the host builder accumulates it, so every array equals the
// host builder's bit for bit.  The boundary tagging and the node-to-element
// incidence stay on the host (integer bookkeeping).
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/tsr_capi.h"
#include "tsr_geom.h"
#include "tsr_internal.h"

namespace {

struct GeomOut {
    double* shape;      // [nv*nv][Ne]
    double* normals;    // [2 nv][Ne]
    double* bmid;       // [4 nv][Ne]
    double* bnrm;       // [4 nv][Ne]
    double* blen;       // [2 nv][Ne]
    double* scv;        // [nv][Ne]
    double* midx;       // [nv][Ne]
    double* midy;       // [nv][Ne]
    double* cent;       // [2][Ne]
};

__global__ void k_element_geometry(int nv, int Mn, int Ne, const double* __restrict__ xy,
                                   const int* __restrict__ el, const unsigned char* __restrict__ isb,
                                   GeomOut o, int* bad)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Ne) return;
    double xv[4], yv[4];
    for (int j = 0; j < nv; ++j) {
        const int v = el[(size_t)j * Ne + k];
        xv[j] = xy[v];
        yv[j] = xy[Mn + v];
    }
    tsr::ElemGeom g;
    if (!tsr::element_geometry(nv, xv, yv, g)) {
        atomicOr(bad, 1);
        return;
    }
    o.cent[k] = g.cx;
    o.cent[Ne + k] = g.cy;
    for (int j = 0; j < nv; ++j) {
        o.scv[(size_t)j * Ne + k] = g.scv[j];
        o.normals[(size_t)(2 * j) * Ne + k] = g.nrm[j][0];
        o.normals[(size_t)(2 * j + 1) * Ne + k] = g.nrm[j][1];
        o.midx[(size_t)j * Ne + k] = g.mid[j][0];
        o.midy[(size_t)j * Ne + k] = g.mid[j][1];
        if (isb[(size_t)j * Ne + k]) {
            for (int s = 0; s < 2; ++s) {
                o.blen[(size_t)(2 * j + s) * Ne + k] = g.blen[j][s];
                for (int d = 0; d < 2; ++d) {
                    o.bmid[(size_t)(4 * j + 2 * s + d) * Ne + k] = g.bmid[j][s][d];
                    o.bnrm[(size_t)(4 * j + 2 * s + d) * Ne + k] = g.bnrm[j][s][d];
                }
            }
        }
    }
    for (int r = 0; r < nv * nv; ++r) o.shape[(size_t)r * Ne + k] = g.sf[r];
}

// CV_area of node i: 0 + its SCV areas over its elements, ascending
__global__ void k_cv_area(int Mn, const int* __restrict__ ptr, const long long* __restrict__ ent,
                          const double* __restrict__ scv, double* __restrict__ cv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Mn) return;
    double a = 0.0;
    for (int p = ptr[i]; p < ptr[i + 1]; ++p) a += scv[ent[p]];
    cv[i] = a;
}

template <typename T>
T* host_zeros(size_t n)
{
    T* p = new (std::nothrow) T[n > 0 ? n : 1];
    if (p) std::memset(p, 0, sizeof(T) * (n > 0 ? n : 1));
    return p;
}

struct DevBuf {
    std::vector<void*> ptrs;
    ~DevBuf()
    {
        for (void* p : ptrs) cudaFree(p);
    }
    template <typename T>
    T* get(size_t n)
    {
        void* p = nullptr;
        if (cudaMalloc(&p, sizeof(T) * (n > 0 ? n : 1)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        cudaMemset(p, 0, sizeof(T) * (n > 0 ? n : 1));
        return static_cast<T*>(p);
    }
};

}  // namespace

extern "C" int tsr_macro_mesh_build_device(int nv, int n_nodes, const double* xy, int n_elems,
                                           const int* elems, int n_bedges, const int* bedges,
                                           const int* macro_bc, macro_mesh_struct* out)
{
    if (!out || !xy || !elems || n_nodes <= 0 || n_elems <= 0 || (nv != 3 && nv != 4) ||
        (n_bedges > 0 && !bedges) || !macro_bc) {
        tsr::set_error("tsr_macro_mesh_build_device: invalid arguments");
        return TSR_ERR_ARG;
    }
    const int Ne = n_elems, Mn = n_nodes;
    for (long i = 0; i < (long)Ne * nv; ++i)
        if (elems[i] < 0 || elems[i] >= Mn) {
            tsr::set_error("tsr_macro_mesh_build_device: invalid arguments");
            return TSR_ERR_ARG;
        }
    std::memset(out, 0, sizeof *out);
    macro_mesh_struct& m = *out;
    m.no_verts = nv;
    m.no_nodes = Mn;
    m.no_elements = Ne;
    const size_t nve = (size_t)nv * Ne;
    m.elements = host_zeros<int>(nve);
    m.nodes = host_zeros<double>(2 * (size_t)Mn);
    m.shape_funcs = host_zeros<double>((size_t)nv * nve);
    m.normals = host_zeros<double>(2 * nve);
    m.boundary_edge_midpts = host_zeros<double>(4 * nve);
    m.boundary_edge_normals = host_zeros<double>(4 * nve);
    m.boundary_edge_lens = host_zeros<double>(2 * nve);
    m.boundary_condition_edges = host_zeros<int>(nve);
    m.CV_area = host_zeros<double>((size_t)Mn);
    m.SCV_area = host_zeros<double>(nve);
    m.midx = host_zeros<double>(nve);
    m.midy = host_zeros<double>(nve);
    m.centroid_elements = host_zeros<double>(2 * (size_t)Ne);
    if (!m.elements || !m.nodes || !m.shape_funcs || !m.normals || !m.boundary_edge_midpts ||
        !m.boundary_edge_normals || !m.boundary_edge_lens || !m.boundary_condition_edges || !m.CV_area ||
        !m.SCV_area || !m.midx || !m.midy || !m.centroid_elements) {
        tsr_macro_mesh_free(out);
        tsr::set_error("tsr_macro_mesh_build_device: out of host memory");
        return TSR_ERR_ALLOC;
    }
    std::memcpy(m.nodes, xy, sizeof(double) * 2 * (size_t)Mn);
    for (int k = 0; k < Ne; ++k)
        for (int v = 0; v < nv; ++v) m.elements[(size_t)v * Ne + k] = elems[(size_t)k * nv + v];
    std::vector<unsigned char> is_bedge(nve, 0);
    if (tsr::macro_bc_edges(nv, Mn, Ne, m.elements, n_bedges, bedges, macro_bc, m.boundary_condition_edges,
                            is_bedge.data())) {
        tsr_macro_mesh_free(out);
        tsr::set_error("tsr_macro_mesh_build_device: boundary edge node out of range");
        return TSR_ERR_BOUNDS;
    }
    // node -> (vertex slot, element) entries, elements ascending
    std::vector<int> ptr((size_t)Mn + 1, 0);
    for (int k = 0; k < Ne; ++k)
        for (int j = 0; j < nv; ++j) ptr[(size_t)m.elements[(size_t)j * Ne + k] + 1]++;
    for (int i = 0; i < Mn; ++i) ptr[(size_t)i + 1] += ptr[i];
    std::vector<long long> ent(nve);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int k = 0; k < Ne; ++k)
        for (int j = 0; j < nv; ++j) ent[(size_t)fill[m.elements[(size_t)j * Ne + k]]++] = (long long)j * Ne + k;

    auto fail = [&](const char* what, cudaError_t e) {
        tsr_macro_mesh_free(out);
        tsr::set_error(std::string("tsr_macro_mesh_build_device: ") + what + ": " + cudaGetErrorString(e));
        return TSR_ERR_CUDA;
    };
    DevBuf d;
    double* d_xy = d.get<double>(2 * (size_t)Mn);
    int* d_el = d.get<int>(nve);
    unsigned char* d_isb = d.get<unsigned char>(nve);
    int* d_ptr = d.get<int>((size_t)Mn + 1);
    long long* d_ent = d.get<long long>(nve);
    int* d_bad = d.get<int>(1);
    GeomOut o;
    o.shape = d.get<double>((size_t)nv * nve);
    o.normals = d.get<double>(2 * nve);
    o.bmid = d.get<double>(4 * nve);
    o.bnrm = d.get<double>(4 * nve);
    o.blen = d.get<double>(2 * nve);
    o.scv = d.get<double>(nve);
    o.midx = d.get<double>(nve);
    o.midy = d.get<double>(nve);
    o.cent = d.get<double>(2 * (size_t)Ne);
    double* d_cv = d.get<double>((size_t)Mn);
    if (!d_xy || !d_el || !d_isb || !d_ptr || !d_ent || !d_bad || !o.shape || !o.normals || !o.bmid || !o.bnrm ||
        !o.blen || !o.scv || !o.midx || !o.midy || !o.cent || !d_cv)
        return fail("device allocation", cudaGetLastError());
    cudaError_t e = cudaSuccess;
    auto h2d = [&](void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess) e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    };
    h2d(d_xy, xy, sizeof(double) * 2 * (size_t)Mn);
    h2d(d_el, m.elements, sizeof(int) * nve);
    h2d(d_isb, is_bedge.data(), nve);
    h2d(d_ptr, ptr.data(), sizeof(int) * ((size_t)Mn + 1));
    h2d(d_ent, ent.data(), sizeof(long long) * nve);
    if (e != cudaSuccess) return fail("copy to the device", e);
    k_element_geometry<<<(Ne + 127) / 128, 128>>>(nv, Mn, Ne, d_xy, d_el, d_isb, o, d_bad);
    k_cv_area<<<(Mn + 127) / 128, 128>>>(Mn, d_ptr, d_ent, o.scv, d_cv);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaDeviceSynchronize()) != cudaSuccess)
        return fail("geometry kernels", e);
    int bad = 0;
    auto d2h = [&](void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess) e = cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost);
    };
    d2h(&bad, d_bad, sizeof(int));
    d2h(m.shape_funcs, o.shape, sizeof(double) * (size_t)nv * nve);
    d2h(m.normals, o.normals, sizeof(double) * 2 * nve);
    d2h(m.boundary_edge_midpts, o.bmid, sizeof(double) * 4 * nve);
    d2h(m.boundary_edge_normals, o.bnrm, sizeof(double) * 4 * nve);
    d2h(m.boundary_edge_lens, o.blen, sizeof(double) * 2 * nve);
    d2h(m.SCV_area, o.scv, sizeof(double) * nve);
    d2h(m.midx, o.midx, sizeof(double) * nve);
    d2h(m.midy, o.midy, sizeof(double) * nve);
    d2h(m.centroid_elements, o.cent, sizeof(double) * 2 * (size_t)Ne);
    d2h(m.CV_area, d_cv, sizeof(double) * (size_t)Mn);
    if (e != cudaSuccess) return fail("copy from the device", e);
    if (bad) {
        tsr_macro_mesh_free(out);
        tsr::set_error("tsr_macro_mesh_build_device: degenerate element");
        return TSR_ERR_ARG;
    }
    return TSR_OK;
}
