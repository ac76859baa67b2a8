// tsr_device.h -- device-side data of one problem and the kernel launchers
// (host-callable).  Only the library's own translation units include this.
#ifndef TSR_DEVICE_H
#define TSR_DEVICE_H

#include <cuda_runtime.h>
#include <cstdint>

namespace tsr {

// Van Genuchten parameters with the derived constants the kernels use.
struct VGPar {
    double Ks, thr, ths, alpha, n, m;
    double dth, coefC, mh;
};

// Micro-cell templates: the reference's one shared micro mesh
// (include/user_data.h:4), or several in the batched form, re-laid out for
// the cell kernel and concatenated; TplDesc holds each template's sizes and
// its offsets into the concatenated arrays.
struct TplDesc {
    int mn, mNe, nb, state;      // nodes, elements, boundary items, shared doubles per cell
    int ev, eg, csr_ptr, csr_ent, node, bitem;   // offsets (elements, nodes, items)
};

struct MicroSet {
    int ntpl;
    int n_bundles;
    int maxc;                    // largest bundle (cells)
    int pad;
    const TplDesc* tpl;          // [ntpl]
    const int* ev;               // 3 per element: vertices
    const double* eg;            // 9 per element: per face j D1, D2, ny
    const int* csr_ptr;          // mn+1 per template
    const int* csr_ent;          // (3e+j)<<1 | (1 if subtracted)
    const int* bnode;            // per node: 1 on the inclusion boundary
    const double* cv;            // per node: CV area
    const double* vec;           // 2 per node (x then y, per template block)
    const int* eb_first;         // per element: first boundary item (template-local)
    const int* eb_count;         // per element
    const int* b_v;              // per item: node (template-local)
    const double* b_n;           // 3 per item: D1, D2, ny of the outward normal
    const long long* cell_off;   // [Ne] first unknown of cell k
    const int* cell_tpl;         // [Ne]
    const struct VGPar* cell_par;   // [Ne] or nullptr (all pB)
    const int* bundle_tpl;       // [n_bundles]
    const int* bundle_first;     // [n_bundles] index into bundle_cells
    const int* bundle_count;     // [n_bundles]
    const int* bundle_cells;     // cell ids, grouped by bundle
};

// Macro mesh in the reference layout plus derived arrays.
struct MacroDev {
    int Mn, Ne, nv;
    int pad;
    const int* elements;    // [nv*Ne]
    const double* sf;       // [nv*nv*Ne]
    const double* normals;  // [2*nv*Ne]
    const double* midx;
    const double* midy;
    const int* bce;         // [nv*Ne]
    const double* blen;     // [2*nv*Ne]
    const double* bmid;     // [4*nv*Ne]
    const double* bnrm;     // [4*nv*Ne]
    const double* scv;      // [nv*Ne]
    const double* cv;       // [Mn]
    const double* cent;     // [2*Ne]
    const unsigned char* dirichlet;  // [Mn]
    const int* csr_ptr;     // [Mn+1]
    const int* csr_ent;     // (16k+slot)<<1 | neg
    const double* keff;     // [4*nk]
    int nk;
    int model_type;
    double keff_first, keff_inv_logr;
    double epsA, inv_Y, Ss, bflux;
};

struct Problem {
    MacroDev M;
    MicroSet m;
    VGPar pA, pB;
    const double* cell_scale;   // [Ne] or nullptr
    int kface;
    int micro_block;            // threads per cell CTA
    size_t micro_smem;          // dynamic shared memory per cell CTA
    int micro_grid;             // persistent grid of the cell kernel
    int misc_slots;             // per-cell scratch slots reserved in shared memory
    double* contrib;            // [16*Ne] macro contributions per element
    int* flag;                  // device word: bit 0 non-finite G
    long long N;
};

// Opt the cell kernel into its dynamic shared memory and report how many
// of its CTAs fit on one SM.  Returns 0 on success.
int configure_cell_kernels(const Problem& P, int* occ);

// Two-scale G (mode 0) or finite-difference Jv (mode 1):
//   mode 0: out = G(u)
//   mode 1: out = (G(u + eps v) - g0) * inv_eps, with epsv = {eps, inv_eps}
//           in device memory
void launch_g(const Problem& P, int mode, const double* u, const double* v, const double* g0,
              const double* epsv, double* out, cudaStream_t s);

// Fixed-order reductions (result written to device scalar *res).
struct RedWork {
    double* partials;       // [nblocks]
    unsigned int* counter;  // one word per concurrent reduction slot
};
int reduction_blocks(long long n);
void launch_dot(const double* x, const double* y, long long n, double* res, RedWork w, cudaStream_t s);
void launch_wsq(const double* x, const double* winv, long long n, double* res, RedWork w, cudaStream_t s);
void launch_vsum(const double* x, long long n, double* res, RedWork w, cudaStream_t s);
// w <- fma(-(*h), vi, w) and *res = dot(w, vnext) (or dot(w, w) if vnext is null)
void launch_mgs(double* w, const double* vi, const double* h, const double* vnext, long long n,
                double* res, RedWork rw, cudaStream_t s);
// *hn = sqrt(*hsq), *ih = 1 / *hn; v = w * (*ih); *res = sum (v winv)^2
void launch_scale_wsq(const double* w, const double* hsq, double* hn, double* ih, double* v,
                      const double* winv, long long n, double* res, RedWork rw, cudaStream_t s);
void launch_scale(const double* x, double a, double* y, long long n, cudaStream_t s);
void launch_winv(const double* u, double rtol, double atol, double* winv, long long n, cudaStream_t s);
// out = u + sum_i c[i] V_i
void launch_combine(const double* u, const double* V, long long ldV, const double* c, int m,
                    double* out, long long n, cudaStream_t s);
// res = sum ((g1 - g0 - sum_i z_i V_i) * dt3 * winv)^2
void launch_err(const double* g1, const double* g0, const double* V, long long ldV, const double* z,
                int mz, double dt3, const double* winv, long long n, double* res, RedWork rw,
                cudaStream_t s);
// number of kernels this library has launched (host counter)
unsigned long long kernel_launches();
void add_launches(int n);
void set_counting(bool on);
// measured FP64 instruction rate of the device (DFMA chains)
int measure_fp64_peak(double* ops_per_s);

// total water content
void launch_water(const Problem& P, const double* u, double* terms, double* res, RedWork rw,
                  cudaStream_t s);

}  // namespace tsr

#endif
