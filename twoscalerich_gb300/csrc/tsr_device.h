// tsr_device.h -- device-side data of one problem and the kernel launchers
// (host-callable).  Only the library's own translation units include this.
#ifndef TSR_DEVICE_H
#define TSR_DEVICE_H

#include <cuda_runtime.h>
#include <cstdint>

struct tsr_mlp;

namespace tsr {

// the closure network's device parameters (tsr_mlp.cu)
const void* mlp_device_weights(const tsr_mlp* m);
const float* mlp_device_params(const tsr_mlp* m);

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
    int kind;                    // 0 micro mesh, 1 learned closure (one unknown per cell)
    int nbn, bnl;                // inclusion-boundary nodes: count, offset into MicroSet::bnl
};

struct MicroSet {
    int ntpl;
    int n_bundles;
    int maxc;                    // largest bundle (cells)
    int pad;
    const TplDesc* tpl;          // [ntpl]
    const int* ev;               // 3 per element: vertices
    const double* eg;            // 6 per element: per face j D1/2, D2/2
    const int* csr_ptr;          // mn+1 per template
    const int* csr_ent;          // (3e+j)<<1 | (1 if subtracted)
    const int* bnode;            // per node: 1 on the inclusion boundary
    const int* bnl;              // per template: its boundary nodes (template-local indices)
    const double* cv;            // per node: CV area
    const double* vec;           // 2 per node (x then y, per template block)
    const int* b_e;              // per item: element (template-local)
    const int* b_v;              // per item: node (template-local)
    const double* b_n;           // 2 per item: D1, D2 of the outward normal
    const long long* cell_off;   // [Ne] first unknown of cell k
    const int* cell_tpl;         // [Ne]
    const struct VGPar* cell_par;   // [Ne] or nullptr (all pB)
    const int* bundle_tpl;       // [n_bundles]
    const int* bundle_first;     // [n_bundles] index into bundle_cells
    const int* bundle_count;     // [n_bundles]
    const int* bundle_cells;     // cell ids, grouped by bundle
    // learned closure
    const int* cell_tpl_full;    // [Ne] micro template of every cell (geometry of learned cells)
    const double* kappa;         // [2 Ne] closure coefficients (kQ, kT) per cell
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
    // ensemble form: nscen scenarios of scen_nodes nodes and scen_cells cells
    int nscen, scen_nodes, scen_cells;
    int pad2;
    const long long* node_off;          // [Mn] unknown of macro node i, or nullptr (identity)
    const struct VGPar* scen_pA;        // [nscen] or nullptr (pA)
    const double* scen_kscale;          // [nscen] or nullptr (1)
};

struct Problem {
    MacroDev M;
    MicroSet m;
    VGPar pA, pB;
    const double* cell_scale;   // [Ne] or nullptr
    int kface;
    int micro_block;            // threads per cell CTA
    size_t micro_smem;          // dynamic shared memory per cell CTA
    int tables_smem;            // 1: the math tables copied into shared memory; 0: read through L1
    int micro_grid;             // persistent grid of the cell kernel
    int misc_slots;             // per-cell scratch slots reserved in shared memory
    double* contrib;            // [16*Ne] macro contributions per element
    double* node_st;            // [2*Mn] macro nodes' storage terms (Cd, den), from the cell kernel
    int* flag;                  // [nscen] device words: bit 0 non-finite G in scenario s
    const int* active;          // [nscen] scenarios to evaluate, or nullptr (all)
    int eps_stride;             // doubles between consecutive scenarios' {eps, 1/eps}
    long long N;
    double* qlog;               // [Ne] exchange inflow of every cell (plain G), or nullptr
};

// Learned-closure update of one step: features of the learned cells, the
// network, the coefficients and the a-posteriori indicator.
struct ClosureDev {
    const void* w;              // bf16 weights (parameter-block indexing)
    const float* p;             // FP32 parameter block (biases)
    double fmu[6], fsd[6];      // feature standardisation
    double ymu[2], ysd[2];      // output de-standardisation
    float zlo[6], zhi[6];       // accepted range of the standardised features
    const int* cells;           // [n] learned cells
    int n;
    int pad;
    double* hist;               // [3 Ne] macro head at the cell centre, last 3 accepted states
    int* hcount;                // [Ne] valid history entries
    double* hcur;               // [Ne] the same at the current state
    double t[4];                // current time and the 3 previous accepted times
    double* kappa;              // [2 Ne]
    const double* aint;         // [ntpl] interior CV area of each template
    int* flags;                 // [Ne] indicator result
    int* nflag;                 // device counter
    double thr;                 // indicator threshold (relative flux change)
    double qfloor;              // flux floor of the relative measure
    const void* w2;             // ensemble: the second network's bf16 weights (or null)
    const float* p2;            // its FP32 parameter block
    double thr_ens;             // threshold on the two networks' inflow difference
};

// Vector segments (one per scenario) for reductions and elementwise work.
// Block b of a segmented launch covers items [start_s + 8192 lb, ...) of
// segment s = blkseg[b], lb = b - block0[s]: chunking is relative to the
// segment, so each segment is reduced in exactly the order it would be alone.
struct SegInfo {
    int nseg;                   // segments
    int nblocks;                // blocks of a launch over all segments
    long long n1;               // length when there is one implicit segment
    const long long* start;     // [nseg+1] or nullptr (one segment [0, n1))
    const int* block0;          // [nseg+1]
    const int* blkseg;          // [nblocks]
    unsigned int* counters;     // [nseg]
    const int* active;          // [nseg] or nullptr (all)
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

// Fixed-order reductions; segment s writes its result to res[s * rstride].
struct RedWork {
    double* partials;       // [blocks]
    unsigned int* counter;  // counters of single-segment launches
};
int reduction_blocks(long long n);
SegInfo single_segment(long long n, RedWork w);
void launch_dot(const double* x, const double* y, const SegInfo& g, double* res, int rstride,
                double* partials, cudaStream_t s);
void launch_wsq(const double* x, const double* winv, const SegInfo& g, double* res, int rstride,
                double* partials, cudaStream_t s);
void launch_vsum(const double* x, const SegInfo& g, double* res, int rstride, double* partials,
                 cudaStream_t s);
// w <- fma(-h_s, vi, w), res_s = dot(w, vnext) (or dot(w, w) if vnext is null),
// h_s = h[s * hstride]
void launch_mgs(double* w, const double* vi, const double* h, int hstride, const double* vnext,
                const SegInfo& g, double* res, int rstride, double* partials, cudaStream_t s);
// hn_s = sqrt(hsq_s), ih_s = 1 / hn_s; v = w * ih_s; res_s = sum (v winv)^2
// (hsq, hn, ih strided by `stride` per segment)
void launch_scale_wsq(const double* w, const double* hsq, double* hn, double* ih, int stride,
                      double* v, const double* winv, const SegInfo& g, double* res, double* partials,
                      cudaStream_t s);
// The Gram-Schmidt block of Arnoldi step j in one cooperative launch
// (results identical to launch_dot + j+1 launch_mgs + launch_scale_wsq):
// column j of scenario s at Hc + s*stride, h_{j+1,j}^2 at hsq, 1/h at ih,
// the weighted norm of v_{j+1} at sv (all strided by `stride`).
struct GsArgs {
    double* w;
    double* V;
    long long ldV;
    double* Hc;
    double* hsq;
    double* ih;
    double* sv;
    int stride;
    int j;
    const double* winv;
    double* partials;           // 2 x pstride (MGS); 2 x parstride (CGS2)
    long long pstride;
    long long parstride;        // CGS2: distance of the two partial buffers
    unsigned int* bar;          // [2] barrier count and generation
    int* err;                   // set if a barrier wait expired
    double* wpart;              // 2 x 128 warp sums of the warp-spread kernel (or null)
};
int gs_fused_grid(int nsm);     // co-resident CTAs of the fused kernel
// the grid barrier's bounded wait run out on purpose (a CTA that never
// arrives); *timed_out = 1 if the wait expired and raised its flag
int barrier_probe(int* timed_out);
cudaError_t launch_gs_fused(const SegInfo& g, const GsArgs& A, int max_grid, cudaStream_t s);
// classical Gram-Schmidt twice: co-resident CTAs for bases up to maxk + 1
// vectors (0: cannot launch), the largest Krylov dimension it takes, launch
int gs_cgs2_grid(int nsm, int maxk);
int gs_cgs2_max_dim();
cudaError_t launch_gs_cgs2(const SegInfo& g, const GsArgs& A, int nsm, cudaStream_t s);

// b = a and d = c on the active segments
void launch_seg_copy2(const double* a, double* b, const double* c, double* d, const SegInfo& g,
                      cudaStream_t s);
// y = x * a_s (a strided)
void launch_seg_scale(const double* x, const double* a, int astride, double* y, const SegInfo& g,
                      cudaStream_t s);
void launch_winv(const double* u, double rtol, double atol, double* winv, const SegInfo& g,
                 cudaStream_t s);
// out = u + sum_{q < m_s} c_s[q] V_q (c_s at c + s * cstride)
void launch_combine(const double* u, const double* V, long long ldV, const double* c, int cstride,
                    const int* m, double* out, const SegInfo& g, cudaStream_t s);
// res_s = sum ((g1 - g0 - sum_{q < mz_s} z_s[q] V_q) * dt3_s * winv)^2
// the step error: D = (g1 - g0 - V z) dt/3 into D (a work vector), then
// the weighted sum of squares of D into res
void launch_err(const double* g1, const double* g0, const double* V, long long ldV, const double* z,
                int zstride, const int* mz, const double* dt3, int dstride, const double* winv,
                const SegInfo& g, double* res, int rstride, double* partials, double* D, cudaStream_t s);

// number of kernels this library has launched (host counter)
unsigned long long kernel_launches();
void add_launches(int n);
void set_counting(bool on);
// measured FP64 instruction rate of the device (DFMA chains)
int measure_fp64_peak(double* ops_per_s);

// per-cell summary (5 doubles: H_c, theta, rate, Q, h(theta)) of state u
// with g = G(u) (g may be null: rate 0) and qlog the cells' exchange inflow
// (may be null: Q 0)
void launch_cell_summary(const Problem& P, const double* u, const double* g, const double* qlog,
                         double* out, cudaStream_t s);
// learned-closure update (coefficients and indicator) and the history push
void launch_closure_update(const Problem& P, const double* u, const ClosureDev& C, cudaStream_t s);
void launch_closure_push(const ClosureDev& C, cudaStream_t s);
// state of a new cell layout: macro part copied, every cell copied or
// converted (micro -> learned: theta from the summary; learned -> micro:
// h(theta) on every node)
void launch_relayout(const Problem& P, int Mn, int Ne, const long long* off_old, const int* learned_old,
                     const long long* off_new, const int* learned_new, const double* summary,
                     const double* u_old, double* u_new, cudaStream_t s);

// water content terms, [macro nodes of s | cells of s] scenario by scenario
// (reduce them with launch_vsum)
void launch_water_terms(const Problem& P, const double* u, double* terms, cudaStream_t s);
// micro-boundary entries of x <- the macro interpolant (solution writer calibration)
void launch_calibrate(const Problem& P, double* x, cudaStream_t s);

}  // namespace tsr

#endif
