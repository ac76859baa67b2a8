// tsr_ctx.cu -- device context, C-ABI entry points and the EXPREM driver.
//
// A context uploads the mesh once (the reference treats the user_data arrays
// as immutable after set-up, include/user_data.h) and owns every device
// buffer the hot path needs, so G, Jv and EXPREM steps allocate nothing.
// The EXPREM step runs its vector work on the GPU (u, G(u), the Krylov basis
// V and all N-length temporaries stay in HBM) and crosses to the host only
// for the (m+1) x m Hessenberg column, a few scalars and phi_1(dt H_m).
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <array>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tsr_capi.h"
#include "tsr_device.h"
#include "tsr_internal.h"
#include "tsr_math.h"

using namespace tsr;

namespace {

constexpr double kKrylovTol = 0.1;   // Krylov error accepted as a fraction of the step tolerance
constexpr int kMaxKrylovCap = 512;

// device scalar slots after each scenario's Hessenberg block
enum { S_HSQ = 0, S_SV, S_ERR, S_DOT, S_BETA2, S_NU2, S_WATER, S_IH, S_EPS, S_IEPS, S_IB, S_COUNT = 16 };

// host state of one scenario's EXPREM integration (the whole problem when
// there is one scenario)
struct ScenState {
    double t = 0.0;
    bool loaded = false;
    bool g0_valid = false;
    int status = 0;              // TSR_OK, or the error that stopped this scenario
    // the step in progress
    double dt = 0.0, beta = 0.0, nu = 0.0, eps = 0.0, errK = 0.0, vnw = 0.0, err = 0.0;
    bool last = false, happy = false, iterating = false;
    int m = 0, maxk = 0;
    int m_prev = 0;              // Krylov dimension of the last accepted step
    std::vector<double> Hm, phi, cv, z;
    int phi_m = 0;               // phi holds phi_1(phi_alpha H_m) for m = phi_m (0: nothing)
    double phi_alpha = 0.0;
    // what limited the last accepted step: its proposed size, the number of
    // halvings because the Krylov space was too small at the largest
    // dimension, the rejected attempts, the error of the accepted attempt,
    // and whether the next step's growth was capped by MaxStepIncFac
    double diag_dt0 = 0.0, diag_err = 0.0;
    int diag_krylov_cuts = 0, diag_rejects = 0, diag_capped = 0, diag_clipped = 0;
};

}  // namespace

struct tsr_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    Problem P{};
    long long N = 0;
    int Mn = 0, Ne = 0;
    std::vector<void*> allocs;
    // work buffers
    double *d_u = nullptr, *d_g0 = nullptr, *d_g1 = nullptr, *d_w = nullptr, *d_unew = nullptr;
    double *d_winv = nullptr, *d_x = nullptr, *d_y = nullptr, *d_z = nullptr, *d_V = nullptr;
    double *d_terms = nullptr, *d_scal = nullptr, *d_coef = nullptr;
    double* h_scal = nullptr;   // pinned mirror of d_scal
    double* h_coef = nullptr;   // pinned coefficients upload
    int* h_flag = nullptr;      // pinned
    RedWork rw{};
    int maxk = 0;
    int ldH = 0;
    // scenarios (one for the plain problem): unknowns [start_s, start_s+1)
    int S = 1;
    std::vector<long long> scen_start;
    SegInfo seg{};               // the unknowns, one segment per scenario
    SegInfo seg_terms{};         // water terms, one segment per scenario
    int* d_active = nullptr;     // [S] scenarios the next launches work on
    int* h_active = nullptr;     // pinned staging of d_active
    std::vector<int> active_now; // what d_active holds
    unsigned int* d_counters = nullptr;
    long long HS = 0;            // doubles per scenario in d_scal (H block + slots)
    int CS = 0;                  // doubles per scenario in d_coef: c | z | dt/3
    int* d_mint = nullptr;       // [2S]: m_s, mz_s
    int* h_mint = nullptr;       // pinned
    double* h_stage = nullptr;   // pinned staging of per-scenario scalars
    // EXPREM state
    std::vector<ScenState> sc;
    const double* last_u0 = nullptr;
    double last_t = -1.0;
    // optional event timing of the kernel classes inside EXPREM steps
    struct ProfEv {
        cudaEvent_t a, b;
        int cat;
        double bytes;
    };
    bool prof = false;
    std::vector<ProfEv> prof_ev;
    size_t prof_used = 0;
    cudaEvent_t marks[16] = {};
    // cell kernel planning (templates, bundles, launch shape)
    std::vector<TplDesc> tpl_host;
    std::vector<int> cell_tpl_host;
    int* d_bundle = nullptr;     // 3 * Ne ints (tpl, first, count) + Ne cell ids
    int nsm = 0, dev_smem = 0;
    int tuned_threads = 0, tuned_budget = 0, tuned_tables = 1;
    // finite-difference step {eps, 1/eps}, staged through pinned memory
    double* h_eps = nullptr;
    // one captured graph per Arnoldi index j, with event nodes timing its
    // Jv and its Gram-Schmidt block
    bool use_graphs = true;
    // dense-output rows calibrated on the device (the solution writer's
    // micro-boundary overwrite) before they are copied out
    bool calibrated_output = false;
    // the Gram-Schmidt block of an Arnoldi step as one cooperative launch
    bool fused_gs = true;
    int gs_grid = 0;
    long long pstride = 0;
    // Gram-Schmidt variant: 0 modified (MGS), 1 classical twice (CGS2, its
    // own fused kernel and partial buffers for j+1 dots per pass)
    int gs_variant = 0;
    int gs2_grid = 0;
    double* d_gs2part = nullptr;
    unsigned int* d_gsbar = nullptr;
    int* d_gserr = nullptr;
    // problems of at most 16 chunks: Gram-Schmidt spread one warp per CTA
    // over the GPU (1) or in one thread-block cluster (0); its warp sums
    int gs_small_warps = 1;
    double* d_gswpart = nullptr;
    std::vector<cudaGraphExec_t> graphs;
    std::vector<std::array<cudaEvent_t, 4>> graph_ev;
    double prof_acc_ms[2] = {0.0, 0.0}, prof_acc_bytes[2] = {0.0, 0.0};
    long long prof_acc_n[2] = {0, 0};
    // learned closure: cell layout that changes between steps
    bool closure = false;
    long long N_cap = 0;                 // unknowns with every cell resolved (buffer capacity)
    int pseudo_tpl = -1;                 // template index of learned cells
    std::vector<int> tpl_full_host;      // [Ne] micro template of every cell
    std::vector<int> learned_host;       // [Ne]
    std::vector<long long> tpl_nodes;    // nodes of each micro template
    long long* d_off[2] = {nullptr, nullptr};
    int* d_learned[2] = {nullptr, nullptr};
    int cur = 0;                         // current layout buffer
    int* d_cell_tpl = nullptr;
    int* d_lcells = nullptr;             // [Ne] learned cells
    int nl = 0;
    double *d_kappa = nullptr, *d_hist = nullptr, *d_hcur = nullptr, *d_summary = nullptr, *d_qlog = nullptr;
    double* d_aint = nullptr;
    int *d_hcount = nullptr, *d_flags = nullptr, *d_nflag = nullptr;
    double thist[3] = {0.0, 0.0, 0.0};
    tsr_mlp* mlp = nullptr;
    tsr_mlp* mlp2 = nullptr;             // ensemble partner of mlp (or null)
    ClosureDev cdev{};
    bool auto_fallback = true;
    // set when a bounded wait of the closure network expired: its tensor
    // memory may have been released under MMAs still in flight, so the
    // context refuses further work (free it and build a new one)
    bool unusable = false;
};

namespace {

const char* cuda_msg(cudaError_t e) { return cudaGetErrorString(e); }

#define CK(call)                                                                 \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if (e_ != cudaSuccess) {                                                 \
            set_error(std::string(#call) + ": " + cuda_msg(e_));                 \
            return TSR_ERR_CUDA;                                                 \
        }                                                                        \
    } while (0)

template <typename T>
int upload(tsr_ctx* c, const T* host, size_t n, const T** out)
{
    void* p = nullptr;
    size_t bytes = sizeof(T) * (n > 0 ? n : 1);
    CK(cudaMalloc(&p, bytes));
    c->allocs.push_back(p);
    if (n > 0 && host) CK(cudaMemcpy(p, host, sizeof(T) * n, cudaMemcpyHostToDevice));
    *out = static_cast<const T*>(p);
    return TSR_OK;
}

int dev_alloc(tsr_ctx* c, size_t bytes, void** out)
{
    void* p = nullptr;
    CK(cudaMalloc(&p, bytes > 0 ? bytes : 8));
    c->allocs.push_back(p);
    *out = p;
    return TSR_OK;
}

VGPar make_vg(const soil_struct& s)
{
    VGPar p;
    p.Ks = s.Ksat;
    p.thr = s.thetar;
    p.ths = s.thetas;
    p.alpha = s.alpha;
    p.n = s.n;
    p.m = s.m;
    p.dth = s.thetas - s.thetar;
    p.coefC = (p.dth * s.m) * s.n;
    p.mh = -0.5 * s.m;
    return p;
}

// Per-node lists of (item, sign) in the order the element loop of the
// CVFE assembly scatters them.
struct Csr {
    std::vector<int> ptr, ent;
};

Csr group_events(int n_nodes, const std::vector<int>& node, const std::vector<int>& code)
{
    Csr c;
    c.ptr.assign((size_t)n_nodes + 1, 0);
    for (int v : node) c.ptr[(size_t)v + 1]++;
    for (int i = 0; i < n_nodes; ++i) c.ptr[(size_t)i + 1] += c.ptr[i];
    std::vector<int> fill(c.ptr.begin(), c.ptr.end() - 1);
    c.ent.assign(node.size(), 0);
    for (size_t e = 0; e < node.size(); ++e) c.ent[(size_t)fill[node[e]]++] = code[e];
    return c;
}


constexpr int kMiscSlots = 32;     // most cells in one bundle

// shared memory of a bundle plan: tables (when copied there), per-cell
// scratch, the largest bundle's state
size_t cell_smem(int slots, size_t state_doubles, bool tables)
{
    return (tables ? sizeof(tsr_math_tables) : 0) + sizeof(double) * 16 * (size_t)slots +
           (sizeof(long long) + 2 * sizeof(int)) * (size_t)slots + sizeof(double) * state_doubles;
}

}  // namespace

namespace tsr {

// Packs cells into bundles (cells of one template, as many as fit in the
// shared-memory budget, at most kMiscSlots), largest templates first, and
// sets the persistent grid of the cell kernel for `threads` per CTA.
int plan_cells(tsr_ctx* c, int threads, int budget, int tables_smem)
{
    Problem& P = c->P;
    // captured graphs hold the old launch shape
    for (auto& g : c->graphs)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    const int ntpl = (int)c->tpl_host.size();
    const size_t fixed = cell_smem(kMiscSlots, 0, tables_smem != 0);
    std::vector<int> per(ntpl, 1);
    size_t max_state = 0;
    for (int t = 0; t < ntpl; ++t) {
        const size_t st = (size_t)c->tpl_host[t].state;
        long long fit = budget > (long long)fixed ? ((long long)budget - (long long)fixed) / (long long)(8 * st) : 0;
        if (fit < 1) fit = 1;
        if (fit > kMiscSlots) fit = kMiscSlots;
        per[t] = (int)fit;
        if ((size_t)per[t] * st > max_state) max_state = (size_t)per[t] * st;
    }
    // scratch slots for the largest bundle only
    const int slots = *std::max_element(per.begin(), per.end());
    const size_t smem = cell_smem(slots, max_state, tables_smem != 0);
    if (smem > (size_t)c->dev_smem) {
        set_error("a micro cell does not fit in shared memory");
        return TSR_ERR_ARG;
    }
    // cells grouped by template, bundles of per[t] cells
    std::vector<std::vector<int>> cells(ntpl);
    for (int k = 0; k < c->Ne; ++k) cells[c->cell_tpl_host[k]].push_back(k);
    std::vector<int> order(ntpl);
    for (int t = 0; t < ntpl; ++t) order[t] = t;
    std::sort(order.begin(), order.end(),
              [&](int a, int b) { return c->tpl_host[a].state > c->tpl_host[b].state; });
    std::vector<int> btpl, bfirst, bcount, bcells;
    for (int t : order) {
        const std::vector<int>& cl = cells[t];
        for (size_t i = 0; i < cl.size(); i += (size_t)per[t]) {
            const int n = (int)std::min((size_t)per[t], cl.size() - i);
            btpl.push_back(t);
            bfirst.push_back((int)bcells.size());
            bcount.push_back(n);
            for (int q = 0; q < n; ++q) bcells.push_back(cl[i + q]);
        }
    }
    const int nbun = (int)btpl.size();
    std::vector<int> buf;
    buf.reserve(3 * (size_t)nbun + bcells.size());
    buf.insert(buf.end(), btpl.begin(), btpl.end());
    buf.insert(buf.end(), bfirst.begin(), bfirst.end());
    buf.insert(buf.end(), bcount.begin(), bcount.end());
    buf.insert(buf.end(), bcells.begin(), bcells.end());
    CK(cudaMemcpy(c->d_bundle, buf.data(), sizeof(int) * buf.size(), cudaMemcpyHostToDevice));
    MicroSet& S = P.m;
    S.n_bundles = nbun;
    S.bundle_tpl = c->d_bundle;
    S.bundle_first = c->d_bundle + nbun;
    S.bundle_count = c->d_bundle + 2 * nbun;
    S.bundle_cells = c->d_bundle + 3 * nbun;
    S.maxc = slots;
    P.misc_slots = slots;
    P.micro_block = threads;
    P.micro_smem = smem;
    P.tables_smem = tables_smem;
    int occ = 1;
    int rc = configure_cell_kernels(P, &occ);
    if (rc) return rc;
    long long grid = (long long)occ * c->nsm;
    P.micro_grid = (int)(grid < nbun ? grid : nbun);
    if (P.micro_grid < 1) P.micro_grid = 1;
    c->tuned_threads = threads;
    c->tuned_budget = budget;
    c->tuned_tables = tables_smem;
    return TSR_OK;
}

}  // namespace tsr

namespace {

int build_problem(tsr_ctx* c, const user_data_struct& ud, const tsr_model_ext* ext)
{
    const macro_mesh_struct& M = ud.macro_mesh;
    if (M.no_verts != 3 && M.no_verts != 4) {
        set_error("macro mesh must have 3 or 4 vertices per element");
        return TSR_ERR_ARG;
    }
    if (ud.model_type < 1 || ud.model_type > 3) {
        set_error("model_type must be 1, 2 or 3");
        return TSR_ERR_ARG;
    }
    const int nv = M.no_verts, Ne = M.no_elements, Mn = M.no_nodes;
    // micro templates: the one micro mesh, or one per cell (batched form)
    const bool batched = ext && ext->n_templates > 0;
    const int ntpl = batched ? ext->n_templates : 1;
    const micro_mesh_struct* tpls = batched ? ext->templates : &ud.micro_mesh;
    if (batched && (!ext->templates || !ext->cell_template)) {
        set_error("batched form needs templates and cell_template");
        return TSR_ERR_ARG;
    }
    for (int t = 0; t < ntpl; ++t) {
        const micro_mesh_struct& m = tpls[t];
        if (m.no_verts != 3) {
            set_error("micro meshes must be triangular");
            return TSR_ERR_ARG;
        }
        for (long long i = 0; i < 3LL * m.no_elements; ++i)
            if (m.elements[i] < 0 || m.elements[i] >= m.no_nodes) {
                set_error("micro element index out of range");
                return TSR_ERR_BOUNDS;
            }
    }
    // scenarios: S disjoint blocks of the macro mesh, unknowns laid out
    // scenario by scenario as [macro nodes of s | cells of s]
    const int nscen = (ext && ext->scenarios > 1) ? ext->scenarios : 1;
    if (Mn % nscen != 0 || Ne % nscen != 0) {
        set_error("the macro mesh is not made of `scenarios` equal blocks");
        return TSR_ERR_ARG;
    }
    const int sn = Mn / nscen, sce = Ne / nscen;
    if (nscen > 1)
        for (int k = 0; k < Ne; ++k)
            for (int j = 0; j < nv; ++j)
                if (M.elements[(size_t)j * Ne + k] / sn != k / sce) {
                    set_error("a macro element links two scenarios");
                    return TSR_ERR_ARG;
                }
    c->S = nscen;
    c->closure = ext && ext->cell_learned;
    if (c->closure && (nscen > 1 || ud.model_type != 3)) {
        set_error("the learned closure needs one scenario and model_type 3");
        return TSR_ERR_ARG;
    }
    c->pseudo_tpl = c->closure ? ntpl : -1;
    c->cell_tpl_host.assign((size_t)Ne, 0);
    c->tpl_full_host.assign((size_t)Ne, 0);
    c->learned_host.assign((size_t)Ne, 0);
    std::vector<long long> cell_off((size_t)Ne), node_off((size_t)Mn);
    c->scen_start.assign((size_t)nscen + 1, 0);
    long long N = 0, Ncap = Mn;
    for (int sc = 0; sc < nscen; ++sc) {
        c->scen_start[sc] = N;
        for (int i = sc * sn; i < (sc + 1) * sn; ++i) node_off[i] = N++;
        for (int k = sc * sce; k < (sc + 1) * sce; ++k) {
            int t = batched ? ext->cell_template[k] : 0;
            if (t < 0 || t >= ntpl) {
                set_error("cell_template out of range");
                return TSR_ERR_BOUNDS;
            }
            const bool lk = c->closure && ext->cell_learned[k];
            c->tpl_full_host[k] = t;
            c->learned_host[k] = lk ? 1 : 0;
            c->cell_tpl_host[k] = lk ? c->pseudo_tpl : t;
            cell_off[k] = N;
            N += lk ? 1 : tpls[t].no_nodes;
            Ncap += tpls[t].no_nodes;
        }
    }
    c->scen_start[nscen] = N;
    c->N_cap = c->closure ? Ncap : N;
    if (Ncap > 0x7fffffffLL) {
        set_error("problem too large for 32-bit indices");
        return TSR_ERR_ARG;
    }
    if (N > 0x7fffffffLL || (long long)Ne * 32 > 0x7fffffffLL) {
        set_error("problem too large for 32-bit indices");
        return TSR_ERR_ARG;
    }
    if (ud.N != 0 && ud.N != (int)N && !(c->closure && ud.N == (int)Ncap)) {
        set_error("user_data.N does not match the meshes");
        return TSR_ERR_ARG;
    }
    for (long long i = 0; i < (long long)nv * Ne; ++i)
        if (M.elements[i] < 0 || M.elements[i] >= Mn) {
            set_error("macro element index out of range");
            return TSR_ERR_BOUNDS;
        }
    c->N = N;
    c->Mn = Mn;
    c->Ne = Ne;
    Problem& P = c->P;
    P.N = N;
    MacroDev& D = P.M;
    D.Mn = Mn;
    D.Ne = Ne;
    D.nv = nv;
    D.model_type = ud.model_type;
    D.nscen = nscen;
    D.scen_nodes = sn;
    D.scen_cells = sce;
    int rc;
    D.node_off = nullptr;
    D.scen_pA = nullptr;
    D.scen_kscale = nullptr;
    if (nscen > 1) {
        if ((rc = upload(c, node_off.data(), node_off.size(), &D.node_off))) return rc;
        if (ext->scen_soilA) {
            std::vector<VGPar> par((size_t)nscen);
            for (int q = 0; q < nscen; ++q) par[q] = make_vg(ext->scen_soilA[q]);
            const VGPar* dp;
            if ((rc = upload(c, par.data(), par.size(), &dp))) return rc;
            D.scen_pA = dp;
        }
        if (ext->scen_keff_scale)
            if ((rc = upload(c, ext->scen_keff_scale, (size_t)nscen, &D.scen_kscale))) return rc;
    }
    const size_t nvNe = (size_t)nv * Ne;
    if ((rc = upload(c, M.elements, nvNe, &D.elements))) return rc;
    if ((rc = upload(c, M.shape_funcs, (size_t)nv * nvNe, &D.sf))) return rc;
    if ((rc = upload(c, M.normals, 2 * nvNe, &D.normals))) return rc;
    if ((rc = upload(c, M.midx, nvNe, &D.midx))) return rc;
    if ((rc = upload(c, M.midy, nvNe, &D.midy))) return rc;
    if ((rc = upload(c, M.boundary_condition_edges, nvNe, &D.bce))) return rc;
    if ((rc = upload(c, M.boundary_edge_lens, 2 * nvNe, &D.blen))) return rc;
    if ((rc = upload(c, M.boundary_edge_midpts, 4 * nvNe, &D.bmid))) return rc;
    if ((rc = upload(c, M.boundary_edge_normals, 4 * nvNe, &D.bnrm))) return rc;
    if ((rc = upload(c, M.SCV_area, nvNe, &D.scv))) return rc;
    if ((rc = upload(c, M.CV_area, (size_t)Mn, &D.cv))) return rc;
    if ((rc = upload(c, M.centroid_elements, 2 * (size_t)Ne, &D.cent))) return rc;
    // Dirichlet nodes: end nodes of type-5 edges
    std::vector<unsigned char> dir((size_t)Mn, 0);
    for (int k = 0; k < Ne; ++k)
        for (int j = 0; j < nv; ++j)
            if (M.boundary_condition_edges[(size_t)j * Ne + k] == TSR_BC_DIRICHLET) {
                dir[M.elements[(size_t)j * Ne + k]] = 1;
                dir[M.elements[(size_t)((j + 1) % nv) * Ne + k]] = 1;
            }
    if ((rc = upload(c, dir.data(), dir.size(), &D.dirichlet))) return rc;
    // macro scatter lists, in the order of the element loop: faces, boundary
    // halves, exchange (slot 16k + s, sign bit 0 = add)
    {
        std::vector<int> node, code;
        node.reserve((size_t)Ne * 16);
        code.reserve((size_t)Ne * 16);
        for (int k = 0; k < Ne; ++k) {
            int v[4];
            for (int j = 0; j < nv; ++j) v[j] = M.elements[(size_t)j * Ne + k];
            for (int j = 0; j < nv; ++j) {
                node.push_back(v[j]);
                code.push_back((16 * k + j) << 1);
                node.push_back(v[(j + 1) % nv]);
                code.push_back(((16 * k + j) << 1) | 1);
            }
            for (int j = 0; j < nv; ++j) {
                int bc = M.boundary_condition_edges[(size_t)j * Ne + k];
                if (bc != TSR_BC_FLUX && bc != TSR_BC_DHDX0 && bc != TSR_BC_DHDY0) continue;
                for (int sh = 0; sh < 2; ++sh) {
                    node.push_back(v[(j + sh) % nv]);
                    code.push_back((16 * k + nv + 2 * j + sh) << 1);
                }
            }
            if (ud.model_type == 3)
                for (int j = 0; j < nv; ++j) {
                    node.push_back(v[j]);
                    code.push_back(((16 * k + 3 * nv + j) << 1) | 1);
                }
        }
        Csr csr = group_events(Mn, node, code);
        if ((rc = upload(c, csr.ptr.data(), csr.ptr.size(), &D.csr_ptr))) return rc;
        if ((rc = upload(c, csr.ent.data(), csr.ent.size(), &D.csr_ent))) return rc;
    }
    const Keff_struct& K = ud.effective_conductivity;
    if (K.no_hvalues < 1 || !K.Keff_values) {
        set_error("empty effective conductivity table");
        return TSR_ERR_ARG;
    }
    D.nk = K.no_hvalues;
    if ((rc = upload(c, K.Keff_values, 4 * (size_t)K.no_hvalues, &D.keff))) return rc;
    D.keff_first = K.logh_first;
    D.keff_inv_logr = 1.0 / K.logr;
    D.epsA = K.epsilonA;
    D.inv_Y = 1.0 / tpls[0].cell_area;
    D.Ss = (ext && ext->specific_storage > 0.0) ? ext->specific_storage : 1e-6;
    D.bflux = ud.boundary_flux;
    P.pA = make_vg(ud.soilA);
    P.pB = make_vg(ud.soilB);
    P.kface = ext ? ext->kface_mode : 0;
    P.cell_scale = nullptr;
    if (ext && ext->cell_scale) {
        if ((rc = upload(c, ext->cell_scale, (size_t)Ne, &P.cell_scale))) return rc;
    }
    // micro templates, concatenated
    MicroSet& S = P.m;
    S.ntpl = ntpl;
    {
        std::vector<int> ev, cptr, cent, bnode, be, bv, bl;
        std::vector<double> eg, cv, vec, bn;
        c->tpl_host.clear();
        for (int t = 0; t < ntpl; ++t) {
            const micro_mesh_struct& m = tpls[t];
            const int mn = m.no_nodes, mNe = m.no_elements;
            TplDesc d{};
            d.mn = mn;
            d.mNe = mNe;
            d.ev = (int)ev.size();
            d.eg = (int)eg.size();
            d.csr_ptr = (int)cptr.size();
            d.csr_ent = (int)cent.size();
            d.node = (int)bnode.size();
            d.bitem = (int)bv.size();
            std::vector<int> node, code;
            for (int e = 0; e < mNe; ++e) {
                int v[3];
                for (int j = 0; j < 3; ++j) {
                    v[j] = m.elements[(size_t)j * mNe + e];
                    ev.push_back(v[j]);
                }
                // face coefficients: (grad h).n_j = D1 (h1 - h0) + D2 (h2 - h0),
                // D_i = sfy_i ny_j + sfx_i nx_j, stored halved (the face
                // conductivity is the mean of two nodal values; the 1/2 is an
                // exact scaling)
                for (int j = 0; j < 3; ++j) {
                    const double nx = m.normals[(size_t)(2 * j) * mNe + e];
                    const double ny = m.normals[(size_t)(2 * j + 1) * mNe + e];
                    for (int i = 1; i <= 2; ++i)
                        eg.push_back(0.5 * std::fma(m.shape_funcs[(size_t)(3 + i) * mNe + e], ny,
                                                    m.shape_funcs[(size_t)i * mNe + e] * nx));
                }
                for (int j = 0; j < 3; ++j) {
                    node.push_back(v[j]);
                    code.push_back((3 * e + j) << 1);
                    node.push_back(v[(j + 1) % 3]);
                    code.push_back(((3 * e + j) << 1) | 1);
                }
                // inclusion-boundary items in assembly order (element,
                // edge, half), each with its element and vertex
                for (int j = 0; j < 3; ++j) {
                    if (m.boundary_edges[(size_t)j * mNe + e] != 1) continue;
                    for (int sh = 0; sh < 2; ++sh) {
                        be.push_back(e);
                        bv.push_back(v[(j + sh) % 3]);
                        const double nbx = m.boundary_edge_normals[(size_t)(4 * j + 2 * sh) * mNe + e];
                        const double nby = m.boundary_edge_normals[(size_t)(4 * j + 2 * sh + 1) * mNe + e];
                        for (int i = 1; i <= 2; ++i)
                            bn.push_back(std::fma(m.shape_funcs[(size_t)(3 + i) * mNe + e], nby,
                                                  m.shape_funcs[(size_t)i * mNe + e] * nbx));
                    }
                }
            }
            d.nb = (int)bv.size() - d.bitem;
            d.state = 4 * mn + 3 * mNe + d.nb;
            Csr csr = group_events(mn, node, code);
            cptr.insert(cptr.end(), csr.ptr.begin(), csr.ptr.end());
            cent.insert(cent.end(), csr.ent.begin(), csr.ent.end());
            d.bnl = (int)bl.size();
            for (int l = 0; l < mn; ++l) {
                bnode.push_back(m.boundary_nodes[l]);
                cv.push_back(m.CV_area[l]);
                if (m.boundary_nodes[l] != 0) bl.push_back(l);
            }
            d.nbn = (int)bl.size() - d.bnl;
            for (int l = 0; l < 2 * mn; ++l) vec.push_back(m.vectors[l]);
            c->tpl_host.push_back(d);
        }
        c->tpl_nodes.assign((size_t)ntpl, 0);
        std::vector<double> aint((size_t)ntpl + 1, 0.0);
        for (int t = 0; t < ntpl; ++t) {
            c->tpl_nodes[t] = tpls[t].no_nodes;
            for (int l = 0; l < tpls[t].no_nodes; ++l)
                if (tpls[t].boundary_nodes[l] != 1) aint[t] += tpls[t].CV_area[l];
        }
        if (c->closure) {
            // learned cells: a template of one unknown and no micro mesh
            TplDesc d{};
            d.mn = 1;
            d.state = 2;
            d.kind = 1;
            c->tpl_host.push_back(d);
        }
        const TplDesc* dt;
        if ((rc = upload(c, c->tpl_host.data(), c->tpl_host.size(), &dt))) return rc;
        S.tpl = dt;
        if ((rc = upload(c, ev.data(), ev.size(), &S.ev))) return rc;
        if ((rc = upload(c, eg.data(), eg.size(), &S.eg))) return rc;
        if ((rc = upload(c, cptr.data(), cptr.size(), &S.csr_ptr))) return rc;
        if ((rc = upload(c, cent.data(), cent.size(), &S.csr_ent))) return rc;
        if ((rc = upload(c, bnode.data(), bnode.size(), &S.bnode))) return rc;
        if (bl.empty()) bl.push_back(0);
        if ((rc = upload(c, bl.data(), bl.size(), &S.bnl))) return rc;
        if ((rc = upload(c, cv.data(), cv.size(), &S.cv))) return rc;
        if ((rc = upload(c, vec.data(), vec.size(), &S.vec))) return rc;
        if ((rc = upload(c, be.data(), be.size(), &S.b_e))) return rc;
        if ((rc = upload(c, bv.data(), bv.size(), &S.b_v))) return rc;
        if ((rc = upload(c, bn.data(), bn.size(), &S.b_n))) return rc;
        void* q;
        for (int b = 0; b < (c->closure ? 2 : 1); ++b) {
            if ((rc = dev_alloc(c, sizeof(long long) * (size_t)(Ne > 0 ? Ne : 1), &q))) return rc;
            c->d_off[b] = (long long*)q;
            if ((rc = dev_alloc(c, sizeof(int) * (size_t)(Ne > 0 ? Ne : 1), &q))) return rc;
            c->d_learned[b] = (int*)q;
        }
        c->cur = 0;
        CK(cudaMemcpy(c->d_off[0], cell_off.data(), sizeof(long long) * (size_t)Ne, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->d_learned[0], c->learned_host.data(), sizeof(int) * (size_t)Ne, cudaMemcpyHostToDevice));
        S.cell_off = c->d_off[0];
        if ((rc = dev_alloc(c, sizeof(int) * (size_t)(Ne > 0 ? Ne : 1), &q))) return rc;
        c->d_cell_tpl = (int*)q;
        CK(cudaMemcpy(c->d_cell_tpl, c->cell_tpl_host.data(), sizeof(int) * (size_t)Ne, cudaMemcpyHostToDevice));
        S.cell_tpl = c->d_cell_tpl;
        if ((rc = upload(c, c->tpl_full_host.data(), c->tpl_full_host.size(), &S.cell_tpl_full))) return rc;
        const double* da;
        if ((rc = upload(c, aint.data(), aint.size(), &da))) return rc;
        c->d_aint = const_cast<double*>(da);
        S.kappa = nullptr;
        if (c->closure) {
            const size_t n2 = 2 * (size_t)Ne;
            if ((rc = dev_alloc(c, sizeof(double) * n2, &q))) return rc;
            c->d_kappa = (double*)q;
            if (ext->closure_coef)
                CK(cudaMemcpy(c->d_kappa, ext->closure_coef, sizeof(double) * n2, cudaMemcpyHostToDevice));
            else
                CK(cudaMemset(c->d_kappa, 0, sizeof(double) * n2));
            S.kappa = c->d_kappa;
            if ((rc = dev_alloc(c, sizeof(double) * 3 * (size_t)Ne, &q))) return rc;
            c->d_hist = (double*)q;
            if ((rc = dev_alloc(c, sizeof(double) * (size_t)Ne, &q))) return rc;
            c->d_hcur = (double*)q;
            if ((rc = dev_alloc(c, sizeof(int) * (size_t)Ne, &q))) return rc;
            c->d_hcount = (int*)q;
            CK(cudaMemset(c->d_hcount, 0, sizeof(int) * (size_t)Ne));
            if ((rc = dev_alloc(c, sizeof(int) * (size_t)Ne, &q))) return rc;
            c->d_flags = (int*)q;
            CK(cudaMemset(c->d_flags, 0, sizeof(int) * (size_t)Ne));
            if ((rc = dev_alloc(c, sizeof(int) * 4, &q))) return rc;
            c->d_nflag = (int*)q;
            if ((rc = dev_alloc(c, sizeof(int) * (size_t)Ne, &q))) return rc;
            c->d_lcells = (int*)q;
            std::vector<int> lc;
            for (int k = 0; k < Ne; ++k)
                if (c->learned_host[k]) lc.push_back(k);
            c->nl = (int)lc.size();
            if (c->nl) CK(cudaMemcpy(c->d_lcells, lc.data(), sizeof(int) * lc.size(), cudaMemcpyHostToDevice));
        }
        if ((rc = dev_alloc(c, sizeof(double) * 5 * (size_t)(Ne > 0 ? Ne : 1), &q))) return rc;
        c->d_summary = (double*)q;
        if ((rc = dev_alloc(c, sizeof(double) * (size_t)(Ne > 0 ? Ne : 1), &q))) return rc;
        c->d_qlog = (double*)q;
        S.cell_par = nullptr;
        if (ext && ext->cell_soilB) {
            std::vector<VGPar> par((size_t)Ne);
            for (int k = 0; k < Ne; ++k) par[k] = make_vg(ext->cell_soilB[k]);
            const VGPar* dp;
            if ((rc = upload(c, par.data(), par.size(), &dp))) return rc;
            S.cell_par = dp;
        }
    }
    void* p;
    if ((rc = dev_alloc(c, sizeof(double) * 16 * (size_t)Ne, &p))) return rc;
    P.contrib = (double*)p;
    CK(cudaMemset(P.contrib, 0, sizeof(double) * 16 * (size_t)Ne));
    if ((rc = dev_alloc(c, sizeof(double) * 2 * (size_t)(c->Mn > 0 ? c->Mn : 1), &p))) return rc;
    P.node_st = (double*)p;
    if ((rc = dev_alloc(c, sizeof(int) * (size_t)(c->S + 3), &p))) return rc;
    P.flag = (int*)p;
    CK(cudaMemset(P.flag, 0, sizeof(int) * (size_t)(c->S + 3)));
    if ((rc = dev_alloc(c, sizeof(int) * (size_t)c->S, &p))) return rc;
    c->d_active = (int*)p;
    CK(cudaMemset(c->d_active, 0, sizeof(int) * (size_t)c->S));
    P.active = (c->S > 1) ? c->d_active : nullptr;
    if ((rc = dev_alloc(c, sizeof(int) * 4 * (size_t)Ne, &p))) return rc;
    c->d_bundle = (int*)p;
    CK(cudaDeviceGetAttribute(&c->dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device));
    // default launch shape: 256 threads (TSR_CELL_THREADS overrides, 64..1024);
    // the smallest shared-memory budget
    // of at least 48 KB that holds one cell of every template
    int threads = 256;
    if (const char* e = std::getenv("TSR_CELL_THREADS")) {
        int v = std::atoi(e);
        if (v >= 64 && v <= 1024 && v % 32 == 0) threads = v;
    }
    return tsr::plan_cells(c, threads, 48 * 1024, 1);
}

// Segments of `start` (S+1 offsets) for the reduction kernels.
int make_seg(tsr_ctx* c, const std::vector<long long>& start, SegInfo* g)
{
    const int S = (int)start.size() - 1;
    std::vector<int> block0((size_t)S + 1, 0), blkseg;
    for (int s = 0; s < S; ++s) {
        const int nb = reduction_blocks(start[(size_t)s + 1] - start[s]);
        block0[(size_t)s + 1] = block0[s] + nb;
        for (int q = 0; q < nb; ++q) blkseg.push_back(s);
    }
    *g = SegInfo{};
    g->nseg = S;
    g->nblocks = block0[S];
    g->n1 = start[S];
    g->counters = c->d_counters;
    if (S == 1) return TSR_OK;    // one segment: no tables, no mask
    int rc;
    if ((rc = upload(c, start.data(), start.size(), &g->start))) return rc;
    if ((rc = upload(c, block0.data(), block0.size(), &g->block0))) return rc;
    if ((rc = upload(c, blkseg.data(), blkseg.size(), &g->blkseg))) return rc;
    g->active = c->d_active;
    return TSR_OK;
}

int alloc_work(tsr_ctx* c, int max_krylov)
{
    const long long N = c->N_cap;   // buffers hold the largest cell layout
    const int S = c->S;
    void* p;
    int rc;
    double** vecs[] = {&c->d_u, &c->d_g0, &c->d_g1, &c->d_w, &c->d_unew, &c->d_winv, &c->d_x, &c->d_y};
    for (double** v : vecs) {
        if ((rc = dev_alloc(c, sizeof(double) * (size_t)N, &p))) return rc;
        *v = (double*)p;
    }
    if ((rc = dev_alloc(c, sizeof(double) * ((size_t)c->Mn + c->Ne), &p))) return rc;
    c->d_terms = (double*)p;
    long long nmin = N;
    for (int s = 0; s < S; ++s) nmin = std::min(nmin, c->scen_start[(size_t)s + 1] - c->scen_start[s]);
    int maxk = max_krylov;
    if (maxk > kMaxKrylovCap) maxk = kMaxKrylovCap;
    if (maxk > nmin) maxk = (int)nmin;
    if (maxk < 0) maxk = 0;
    c->maxk = maxk;
    c->ldH = maxk + 1;
    const int mk1 = maxk > 0 ? maxk : 1;
    if (maxk > 0) {
        if ((rc = dev_alloc(c, sizeof(double) * (size_t)N * (size_t)(maxk + 1), &p))) return rc;
        c->d_V = (double*)p;
    }
    // H block, the fixed slots, then the weighted norm of v_{j+1} for every j
    c->HS = (long long)c->ldH * mk1 + S_COUNT + mk1;
    const size_t nscal = (size_t)c->HS * (size_t)S;
    if ((rc = dev_alloc(c, sizeof(double) * nscal, &p))) return rc;
    c->d_scal = (double*)p;
    CK(cudaMemset(c->d_scal, 0, sizeof(double) * nscal));
    c->P.eps_stride = (int)c->HS;
    c->CS = 2 * mk1 + 4;
    if ((rc = dev_alloc(c, sizeof(double) * (size_t)c->CS * S, &p))) return rc;
    c->d_coef = (double*)p;
    CK(cudaMemset(c->d_coef, 0, sizeof(double) * (size_t)c->CS * S));
    if ((rc = dev_alloc(c, sizeof(int) * 2 * (size_t)S, &p))) return rc;
    c->d_mint = (int*)p;
    if ((rc = dev_alloc(c, sizeof(unsigned int) * (size_t)(S + 3), &p))) return rc;
    c->d_counters = (unsigned int*)p;
    CK(cudaMemset(c->d_counters, 0, sizeof(unsigned int) * (size_t)(S + 3)));
    c->rw.counter = c->d_counters;
    if ((rc = make_seg(c, c->scen_start, &c->seg))) return rc;
    std::vector<long long> tstart((size_t)S + 1);
    for (int s = 0; s <= S; ++s) tstart[s] = (long long)s * ((c->Mn + c->Ne) / S);
    if ((rc = make_seg(c, tstart, &c->seg_terms))) return rc;
    const int nb = std::max(std::max(c->seg.nblocks, c->seg_terms.nblocks),
                            reduction_blocks(std::max(N, (long long)c->Mn + c->Ne)));
    // two partial buffers: the fused Gram-Schmidt kernel alternates them
    if ((rc = dev_alloc(c, sizeof(double) * 2 * (size_t)nb, &p))) return rc;
    c->rw.partials = (double*)p;
    c->pstride = nb;
    if ((rc = dev_alloc(c, sizeof(unsigned int) * 4, &p))) return rc;
    c->d_gsbar = (unsigned int*)p;
    CK(cudaMemset(c->d_gsbar, 0, sizeof(unsigned int) * 4));
    if ((rc = dev_alloc(c, sizeof(int) * 2, &p))) return rc;
    c->d_gserr = (int*)p;
    if ((rc = dev_alloc(c, sizeof(double) * 256, &p))) return rc;
    c->d_gswpart = (double*)p;
    CK(cudaMemset(c->d_gserr, 0, sizeof(int) * 2));
    c->gs_grid = gs_fused_grid(c->nsm);
    if (c->gs_grid < 1) c->fused_gs = false;
    if (const char* e = std::getenv("TSR_FUSED_GS"))
        if (e[0] == '0') c->fused_gs = false;
    CK(cudaMallocHost(&c->h_scal, sizeof(double) * (size_t)c->ldH * 2));
    CK(cudaMallocHost(&c->h_coef, sizeof(double) * (size_t)c->CS * S));
    CK(cudaMallocHost(&c->h_flag, sizeof(int) * (size_t)S));
    CK(cudaMallocHost(&c->h_eps, sizeof(double) * 3 * (size_t)S));
    CK(cudaMallocHost(&c->h_active, sizeof(int) * (size_t)S));
    CK(cudaMallocHost(&c->h_mint, sizeof(int) * 2 * (size_t)S));
    CK(cudaMallocHost(&c->h_stage, sizeof(double) * ((size_t)c->ldH * mk1 + mk1 + 4) * S));
    std::memset(c->h_eps, 0, sizeof(double) * 3 * (size_t)S);
    std::memset(c->h_coef, 0, sizeof(double) * (size_t)c->CS * S);
    std::memset(c->h_mint, 0, sizeof(int) * 2 * (size_t)S);
    c->active_now.assign((size_t)S, 0);
    c->graphs.assign((size_t)mk1, nullptr);
    c->graph_ev.resize((size_t)mk1);
    for (auto& a : c->graph_ev) a.fill(nullptr);
    c->sc.assign((size_t)S, ScenState{});
    for (auto& q : c->sc) {
        q.Hm.assign((size_t)c->ldH * mk1, 0.0);
        q.phi.assign((size_t)mk1 * mk1, 0.0);
        q.cv.assign((size_t)mk1 + 1, 0.0);
        q.z.assign((size_t)mk1 + 2, 0.0);
    }
    return TSR_OK;
}

// per-scenario non-finite flags of the last G launches
int read_flags(tsr_ctx* c)
{
    CK(cudaMemcpyAsync(c->h_flag, c->P.flag, sizeof(int) * (size_t)c->S, cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return TSR_OK;
}

int reset_flag(tsr_ctx* c)
{
    CK(cudaMemsetAsync(c->P.flag, 0, sizeof(int) * (size_t)c->S, c->stream));
    return TSR_OK;
}

double* scal_slot(tsr_ctx* c, int slot, int scen = 0)
{
    return c->d_scal + (size_t)c->HS * (size_t)scen + (size_t)c->ldH * (size_t)(c->maxk > 0 ? c->maxk : 1) +
           slot;
}

int fetch_scalar(tsr_ctx* c, int slot, double* out)
{
    CK(cudaMemcpyAsync(c->h_scal, scal_slot(c, slot), sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *out = c->h_scal[0];
    return TSR_OK;
}

// slot `slot` of every scenario into out[S]
int fetch_scalars(tsr_ctx* c, int slot, double* out)
{
    CK(cudaMemcpy2DAsync(c->h_stage, sizeof(double), scal_slot(c, slot), sizeof(double) * (size_t)c->HS,
                         sizeof(double), (size_t)c->S, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    std::memcpy(out, c->h_stage, sizeof(double) * (size_t)c->S);
    return TSR_OK;
}

// the scenario mask of the next launches (no copy when unchanged); every
// launching path passes through here, so a context marked unusable stops
// here before it launches anything
int set_active(tsr_ctx* c, const std::vector<int>& on)
{
    if (c->unusable) {
        set_error("context unusable after an expired tensor-core wait; free it and create a new one");
        return TSR_ERR_TIMEOUT;
    }
    if (c->S == 1 || on == c->active_now) return TSR_OK;
    CK(cudaStreamSynchronize(c->stream));   // the staging buffer may still be in flight
    for (int s = 0; s < c->S; ++s) c->h_active[s] = on[s];
    CK(cudaMemcpyAsync(c->d_active, c->h_active, sizeof(int) * (size_t)c->S, cudaMemcpyHostToDevice,
                       c->stream));
    c->active_now = on;
    return TSR_OK;
}

// every scenario active (the G, Jv and water entry points work on all)
int all_active(tsr_ctx* c) { return set_active(c, std::vector<int>((size_t)c->S, 1)); }

// {eps, 1/eps, 1/beta} of every scenario into its scalar slots
// (the caller has synchronised the stream before writing h_eps)
int upload_eps(tsr_ctx* c)
{
    CK(cudaMemcpy2DAsync(scal_slot(c, S_EPS), sizeof(double) * (size_t)c->HS, c->h_eps, 3 * sizeof(double),
                         3 * sizeof(double), (size_t)c->S, cudaMemcpyHostToDevice, c->stream));
    return TSR_OK;
}

// one finite-difference step for every scenario
int set_eps(tsr_ctx* c, double eps)
{
    CK(cudaStreamSynchronize(c->stream));
    for (int s = 0; s < c->S; ++s) {
        c->h_eps[3 * s] = eps;
        c->h_eps[3 * s + 1] = 1.0 / eps;
        c->h_eps[3 * s + 2] = 0.0;
    }
    return upload_eps(c);
}

constexpr size_t kProfMax = 16384;

// open an event pair of category cat (0: G / Jv, 1: Gram-Schmidt block)
int prof_begin(tsr_ctx* c, int cat, double bytes)
{
    if (!c->prof) return -1;
    if (c->prof_used >= kProfMax) return -1;
    if (c->prof_used == c->prof_ev.size()) {
        tsr_ctx::ProfEv e{};
        if (cudaEventCreate(&e.a) != cudaSuccess || cudaEventCreate(&e.b) != cudaSuccess) return -1;
        c->prof_ev.push_back(e);
    }
    tsr_ctx::ProfEv& e = c->prof_ev[c->prof_used];
    e.cat = cat;
    e.bytes = bytes;
    cudaEventRecord(e.a, c->stream);
    return (int)c->prof_used++;
}

void prof_end(tsr_ctx* c, int id)
{
    if (id >= 0) cudaEventRecord(c->prof_ev[(size_t)id].b, c->stream);
}

// algorithmic bytes of one G (u in, g out) or one Jv (u, v, g0 in, w out)
// plus the macro geometry each evaluation must read
double g_bytes(const tsr_ctx* c, bool jv)
{
    const double nv = c->P.M.nv;
    const double per_elem = 4 * nv + 8 * nv * nv + 16 * nv + 16 * nv + 8 * nv + 16 + 4 * nv +
                            (c->P.cell_scale ? 8 : 0);
    return (jv ? 32.0 : 16.0) * (double)c->N + per_elem * c->Ne + 8.0 * c->Mn;
}

}  // namespace

// ---- C-ABI ----------------------------------------------------------------

extern "C" tsr_ctx* tsr_init(const user_data_struct* ud, const tsr_model_ext* ext, void* stream,
                             int max_krylov)
{
    if (!ud) {
        set_error("tsr_init: user_data is NULL");
        return nullptr;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev < 1) {
        set_error(std::string("tsr_init: no CUDA device: ") + cudaGetErrorString(e));
        return nullptr;
    }
    tsr_ctx* c = new tsr_ctx();
    cudaGetDevice(&c->device);
    if (stream) {
        c->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
            set_error("tsr_init: cannot create stream");
            delete c;
            return nullptr;
        }
        c->own_stream = true;
    }
    int rc = build_problem(c, *ud, ext);
    if (rc == TSR_OK) rc = alloc_work(c, max_krylov);
    if (rc == TSR_OK && cudaDeviceSynchronize() != cudaSuccess) {
        set_error("tsr_init: device error during set-up");
        rc = TSR_ERR_CUDA;
    }
    if (rc != TSR_OK) {
        tsr_free(c);
        return nullptr;
    }
    return c;
}

extern "C" void tsr_free(tsr_ctx* c)
{
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& e : c->prof_ev) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    for (auto& e : c->marks)
        if (e) cudaEventDestroy(e);
    for (auto& g : c->graphs)
        if (g) cudaGraphExecDestroy(g);
    for (auto& a : c->graph_ev)
        for (auto& e : a)
            if (e) cudaEventDestroy(e);
    if (c->h_eps) cudaFreeHost(c->h_eps);
    if (c->h_active) cudaFreeHost(c->h_active);
    if (c->h_mint) cudaFreeHost(c->h_mint);
    if (c->h_stage) cudaFreeHost(c->h_stage);
    for (void* p : c->allocs) cudaFree(p);
    if (c->h_scal) cudaFreeHost(c->h_scal);
    if (c->h_coef) cudaFreeHost(c->h_coef);
    if (c->h_flag) cudaFreeHost(c->h_flag);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

extern "C" void* tsr_stream(tsr_ctx* c) { return c ? (void*)c->stream : nullptr; }
extern "C" int tsr_num_unknowns(tsr_ctx* c) { return c ? (int)c->N : 0; }

extern "C" int tsr_g_eval_device(tsr_ctx* c, const double* d_u, double* d_g)
{
    if (!c || !d_u || !d_g) return TSR_ERR_ARG;
    int rc = all_active(c);
    if (rc) return rc;
    launch_g(c->P, 0, d_u, nullptr, nullptr, nullptr, d_g, c->stream);
    CK(cudaGetLastError());
    return TSR_OK;
}

extern "C" int tsr_jv_device(tsr_ctx* c, const double* d_u, const double* d_g0, const double* d_v,
                             double eps, double* d_w)
{
    if (!c || !d_u || !d_g0 || !d_v || !d_w || !(eps != 0.0)) return TSR_ERR_ARG;
    int rc = set_eps(c, eps);
    if (rc == TSR_OK) rc = all_active(c);
    if (rc) return rc;
    launch_g(c->P, 1, d_u, d_v, d_g0, scal_slot(c, S_EPS), d_w, c->stream);
    CK(cudaGetLastError());
    return TSR_OK;
}

extern "C" int tsr_g_eval(tsr_ctx* c, const double* u, double* g)
{
    if (!c || !u || !g) return TSR_ERR_ARG;
    const size_t bytes = sizeof(double) * (size_t)c->N;
    int rc;
    if ((rc = all_active(c))) return rc;
    if ((rc = reset_flag(c))) return rc;
    CK(cudaMemcpyAsync(c->d_x, u, bytes, cudaMemcpyHostToDevice, c->stream));
    launch_g(c->P, 0, c->d_x, nullptr, nullptr, nullptr, c->d_y, c->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(g, c->d_y, bytes, cudaMemcpyDeviceToHost, c->stream));
    if ((rc = read_flags(c))) return rc;
    for (int q = 0; q < c->S; ++q)
        if (c->h_flag[q]) {
            set_error("G: non-finite value");
            return TSR_ERR_NAN;
        }
    return TSR_OK;
}

extern "C" int tsr_jv(tsr_ctx* c, const double* u, const double* g0, const double* v, double eps,
                      double* w)
{
    if (!c || !u || !g0 || !v || !w || !(eps != 0.0)) return TSR_ERR_ARG;
    const size_t bytes = sizeof(double) * (size_t)c->N;
    CK(cudaMemcpyAsync(c->d_x, u, bytes, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_w, v, bytes, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_g1, g0, bytes, cudaMemcpyHostToDevice, c->stream));
    int rc = set_eps(c, eps);
    if (rc == TSR_OK) rc = all_active(c);
    if (rc) return rc;
    launch_g(c->P, 1, c->d_x, c->d_w, c->d_g1, scal_slot(c, S_EPS), c->d_y, c->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(w, c->d_y, bytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return TSR_OK;
}

extern "C" int tsr_water_content(tsr_ctx* c, const double* u, double* water)
{
    if (!c || !u || !water) return TSR_ERR_ARG;
    CK(cudaMemcpyAsync(c->d_x, u, sizeof(double) * (size_t)c->N, cudaMemcpyHostToDevice, c->stream));
    launch_water_terms(c->P, c->d_x, c->d_terms, c->stream);
    launch_vsum(c->d_terms, single_segment((long long)c->Mn + c->Ne, c->rw), scal_slot(c, S_WATER), 1,
                c->rw.partials, c->stream);
    CK(cudaGetLastError());
    return fetch_scalar(c, S_WATER, water);
}

extern "C" int tsr_ensemble_water(tsr_ctx* c, const double* u, double* water)
{
    if (!c || !u || !water) return TSR_ERR_ARG;
    int rc;
    if ((rc = set_active(c, std::vector<int>((size_t)c->S, 1)))) return rc;
    CK(cudaMemcpyAsync(c->d_x, u, sizeof(double) * (size_t)c->N, cudaMemcpyHostToDevice, c->stream));
    launch_water_terms(c->P, c->d_x, c->d_terms, c->stream);
    // per-scenario sums, scenario s into its S_WATER slot
    launch_vsum(c->d_terms, c->seg_terms, scal_slot(c, S_WATER), (int)c->HS, c->rw.partials, c->stream);
    CK(cudaGetLastError());
    return fetch_scalars(c, S_WATER, water);
}

extern "C" int tsr_num_scenarios(tsr_ctx* c) { return c ? c->S : 0; }

extern "C" int tsr_scenario_range(tsr_ctx* c, int s, long long* first, long long* count)
{
    if (!c || s < 0 || s >= c->S || !first || !count) return TSR_ERR_ARG;
    *first = c->scen_start[s];
    *count = c->scen_start[(size_t)s + 1] - c->scen_start[s];
    return TSR_OK;
}

extern "C" int tsr_dot(tsr_ctx* c, const double* x, const double* y, int n, double* out)
{
    if (!c || !x || !y || !out || n < 0 || n > c->N) return TSR_ERR_ARG;
    const size_t bytes = sizeof(double) * (size_t)n;
    CK(cudaMemcpyAsync(c->d_x, x, bytes, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_y, y, bytes, cudaMemcpyHostToDevice, c->stream));
    launch_dot(c->d_x, c->d_y, single_segment(n, c->rw), scal_slot(c, S_DOT), 1, c->rw.partials, c->stream);
    CK(cudaGetLastError());
    return fetch_scalar(c, S_DOT, out);
}

// ---- EXPREM ------------------------------------------------------------------
// The same algorithm, operation for operation, as the oracle's
// oracle_exprem_step (the reference's exprem, include/main.h:29-32, whose body
// is not in its tree), run for the S scenarios of
// a context in lockstep: each launch covers the scenarios that need it (a
// device mask), every reduction is segmented per scenario in the
// single-problem order, and each scenario keeps its own step size, Krylov
// dimension and statistics.  With one scenario this is the reference's
// one-step exprem.

extern "C" int tsr_exprem_load(tsr_ctx* c, const double* u_host, double t)
{
    if (!c || !u_host) return TSR_ERR_ARG;
    CK(cudaMemcpyAsync(c->d_u, u_host, sizeof(double) * (size_t)c->N, cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (auto& q : c->sc) {
        q.loaded = true;
        q.t = t;
        q.g0_valid = false;
        q.status = TSR_OK;
    }
    return TSR_OK;
}

extern "C" int tsr_ensemble_load(tsr_ctx* c, const double* u_host, const double* t)
{
    if (!c || !u_host || !t) return TSR_ERR_ARG;
    CK(cudaMemcpyAsync(c->d_u, u_host, sizeof(double) * (size_t)c->N, cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int q = 0; q < c->S; ++q) {
        ScenState& z = c->sc[q];
        z.loaded = true;
        z.t = t[q];
        z.g0_valid = false;
    }
    return TSR_OK;
}

extern "C" int tsr_exprem_store(tsr_ctx* c, double* u_host)
{
    if (!c || !u_host || !c->sc[0].loaded) return TSR_ERR_ARG;
    CK(cudaMemcpyAsync(u_host, c->d_u, sizeof(double) * (size_t)c->N, cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return TSR_OK;
}

namespace {

int phi_host(tsr_ctx* c, ScenState& z, double alpha, int m)
{
    int rc = phipade_host(z.phi.data(), z.Hm.data(), alpha, m, c->ldH, c->maxk);
    if (rc) set_error("phipade: singular Pade denominator");
    z.phi_m = rc ? 0 : m;
    z.phi_alpha = alpha;
    return rc;
}

// phi_1(dt H_m) for the Krylov dimensions that the column tests of one
// batch of Arnoldi steps may reach, each scenario up to its happy breakdown
// or its largest dimension.  They are independent, so they are evaluated
// side by side on the host's threads (phipade_host is re-entrant); each is
// the value phi_host would give, and the tests take them in their
// sequential order.
struct PhiJob {
    int q, m, rc;
    size_t off;
};

void phi_batch(tsr_ctx* c, const std::vector<int>& arn, int j, int nb, size_t row, int min_krylov,
               std::vector<PhiJob>& jobs, std::vector<int>& slot, std::vector<double>& buf)
{
    jobs.clear();
    slot.assign((size_t)c->S * (size_t)nb, -1);     // (scenario, m - 1 - j) -> job
    const int ldH = c->ldH;
    const size_t blk = (size_t)c->maxk * (size_t)c->maxk;
    for (int q = 0; q < c->S; ++q) {
        if (!arn[q]) continue;
        ScenState& z = c->sc[q];
        for (int jj = j; jj < j + nb; ++jj) {
            const double* col = c->h_stage + (size_t)q * row + (size_t)(jj - j) * ldH;
            double hs = 0.0;
            for (int i = 0; i <= jj; ++i) {
                z.Hm[(size_t)jj * ldH + i] = col[i];
                hs = std::fma(col[i], col[i], hs);
            }
            const double hn = col[jj + 1];
            z.Hm[(size_t)jj * ldH + jj + 1] = hn;
            const int m = jj + 1;
            if (!(hn > 1e-12 * std::sqrt(std::fma(hn, hn, hs)))) break;
            if (!(m < min_krylov && m < z.maxk)) {
                slot[(size_t)q * nb + (size_t)(jj - j)] = (int)jobs.size();
                jobs.push_back({q, m, 0, 0});
            }
            if (m >= z.maxk) break;
        }
    }
    for (size_t k = 0; k < jobs.size(); ++k) jobs[k].off = k * blk;
    if (buf.size() < jobs.size() * blk) buf.resize(jobs.size() * blk);
    const long n = (long)jobs.size();
#pragma omp parallel for schedule(dynamic, 1) if (n > 1)
    for (long k = n - 1; k >= 0; --k) {          // largest dimensions first
        PhiJob& J = jobs[(size_t)k];
        ScenState& z = c->sc[J.q];
        J.rc = phipade_host(buf.data() + J.off, z.Hm.data(), z.dt, J.m, c->ldH, c->maxk);
    }
}

// The kernels of Arnoldi step j for every active scenario: w = J v_j
// (finite differences), modified Gram-Schmidt against v_0..v_j,
// h_{j+1,j} = ||w||, v_{j+1} = w / h_{j+1,j} and the weighted norm of
// v_{j+1}.  ev (4 events or null) brackets the Jv and the Gram-Schmidt
// block; otherwise the profiling pool does.  3 kernels (fused Gram-Schmidt)
// or j + 6.
void arnoldi_kernels(tsr_ctx* c, int j, cudaEvent_t* ev, double frac)
{
    const long long N = c->N;
    cudaStream_t s = c->stream;
    double* V = c->d_V;
    const int HS = (int)c->HS;
    double* Hc = c->d_scal + (size_t)j * c->ldH;   // scenario q's column at Hc + q HS
    const SegInfo& g = c->seg;
    double* part = c->rw.partials;
    int pe = -1;
    // inside a capture, only "external" records become event-record nodes
    if (ev) cudaEventRecordWithFlags(ev[0], s, cudaEventRecordExternal);
    else pe = prof_begin(c, 0, frac * g_bytes(c, true));
    launch_g(c->P, 1, c->d_u, V + (size_t)j * N, c->d_g0, scal_slot(c, S_EPS), c->d_w, s);
    if (ev) {
        cudaEventRecordWithFlags(ev[1], s, cudaEventRecordExternal);
        cudaEventRecordWithFlags(ev[2], s, cudaEventRecordExternal);
    } else {
        prof_end(c, pe);
        pe = prof_begin(c, 1, frac * 8.0 * (double)N * (double)(j + 3));   // algorithmic minimum
    }
    if (c->gs_variant == 1) {
        GsArgs A{};
        A.w = c->d_w;
        A.V = V;
        A.ldV = N;
        A.Hc = Hc;
        A.hsq = scal_slot(c, S_HSQ);
        A.ih = scal_slot(c, S_IH);
        A.sv = scal_slot(c, S_COUNT + j);
        A.stride = HS;
        A.j = j;
        A.winv = c->d_winv;
        A.partials = c->d_gs2part;
        A.pstride = c->pstride;
        A.parstride = (long long)(c->maxk + 1) * c->pstride;
        A.bar = c->d_gsbar;
        A.err = c->d_gserr;
        launch_gs_cgs2(g, A, c->gs2_grid, s);
    } else if (c->fused_gs) {
        GsArgs A{};
        A.w = c->d_w;
        A.V = V;
        A.ldV = N;
        A.Hc = Hc;
        A.hsq = scal_slot(c, S_HSQ);
        A.ih = scal_slot(c, S_IH);
        A.sv = scal_slot(c, S_COUNT + j);
        A.stride = HS;
        A.j = j;
        A.winv = c->d_winv;
        A.partials = part;
        A.pstride = c->pstride;
        A.bar = c->d_gsbar;
        A.err = c->d_gserr;
        A.wpart = c->gs_small_warps ? c->d_gswpart : nullptr;
        // the grid barrier's counters: every completed barrier leaves the
        // count at 0 and only advances the generation, so they need no
        // reset between launches (only after an expired wait, below)
        launch_gs_fused(g, A, c->gs_grid, s);
    } else {
        launch_dot(c->d_w, V, g, Hc, HS, part, s);
        for (int i = 0; i <= j; ++i) {
            const double* vnext = (i < j) ? V + (size_t)(i + 1) * N : nullptr;
            double* res = (i < j) ? Hc + i + 1 : scal_slot(c, S_HSQ);
            launch_mgs(c->d_w, V + (size_t)i * N, Hc + i, HS, vnext, g, res, HS, part, s);
        }
        launch_scale_wsq(c->d_w, scal_slot(c, S_HSQ), Hc + j + 1, scal_slot(c, S_IH), HS,
                         V + (size_t)(j + 1) * N, c->d_winv, g, scal_slot(c, S_COUNT + j), part, s);
    }
    if (ev) cudaEventRecordWithFlags(ev[3], s, cudaEventRecordExternal);
    else prof_end(c, pe);
}

struct RoundIO {
    double tend;
    const double* tspan;
    double* const* solns;              // [S] rows of tspan solutions, or null
    const exprem_options_struct* opt;
    exprem_stats_struct* st;           // [S]
};

// One accepted step for every scenario of `part`.  A scenario that fails
// records its status and leaves the round; a CUDA error ends the round.
int exprem_round(tsr_ctx* c, const std::vector<int>& part, const RoundIO& io)
{
    thread_local std::vector<PhiJob> phi_jobs;
    thread_local std::vector<int> phi_slot;
    thread_local std::vector<double> phi_buf;
    const int S = c->S;
    const exprem_options_struct* opt = io.opt;
    cudaStream_t s = c->stream;
    const long long N = c->N;
    double* V = c->d_V;
    const int ldH = c->ldH;
    const int HS = (int)c->HS;
    const int mk1 = c->maxk > 0 ? c->maxk : 1;
    int rc;
    auto Ns = [&](int q) { return c->scen_start[(size_t)q + 1] - c->scen_start[q]; };
    auto fail = [&](int q, int code, const char* msg) {
        c->sc[q].status = code;
        set_error(msg);
    };
    auto mask_of = [&](const std::vector<int>& set) {
        std::vector<int> m((size_t)S, 0);
        for (int q : set) m[q] = 1;
        return m;
    };
    // step set-up
    std::vector<int> live;
    for (int q : part) {
        ScenState& z = c->sc[q];
        exprem_stats_struct& st = io.st[q];
        z.status = TSR_OK;
        if (z.t == 0.0) {
            st.NumSteps = 0;
            st.FuncEvals = 0;
            st.CurrentStep = opt->InitStep;
            st.CurrentKryDim = 0;
            st.CurrentTime = 0.0;
            z.g0_valid = false;
        }
        if (st.NumSteps >= opt->MaxNumSteps) {
            fail(q, TSR_ERR_MAXSTEPS, "MaxNumSteps reached");
            continue;
        }
        long long mq = std::min((long long)opt->MaxKrylov, Ns(q));
        z.maxk = (int)std::min(mq, (long long)c->maxk);
        z.dt = st.CurrentStep;
        if (z.dt > opt->MaxStep) z.dt = opt->MaxStep;
        z.last = false;
        z.diag_dt0 = z.dt;
        z.diag_krylov_cuts = 0;
        z.diag_rejects = 0;
        z.diag_clipped = 0;
        if (z.t + z.dt >= io.tend) {
            z.dt = io.tend - z.t;
            z.last = true;
            z.diag_clipped = 1;
        }
        live.push_back(q);
    }
    // G(u) where the previous step did not leave it
    std::vector<int> need;
    for (int q : live)
        if (!c->sc[q].g0_valid) need.push_back(q);
    if (!need.empty()) {
        if ((rc = set_active(c, mask_of(need)))) return rc;
        if ((rc = reset_flag(c))) return rc;
        int pe = prof_begin(c, 0, g_bytes(c, false) * need.size() / S);
        launch_g(c->P, 0, c->d_u, nullptr, nullptr, nullptr, c->d_g0, s);
        prof_end(c, pe);
        CK(cudaGetLastError());
        if ((rc = read_flags(c))) return rc;
        std::vector<int> keep;
        for (int q : live) {
            ScenState& z = c->sc[q];
            if (!z.g0_valid) {
                io.st[q].FuncEvals++;
                if (c->h_flag[q]) {
                    fail(q, TSR_ERR_GFUNC, "G(u) non-finite at the current state");
                    continue;
                }
                z.g0_valid = true;
            }
            keep.push_back(q);
        }
        live.swap(keep);
    }
    if (live.empty()) return TSR_OK;
    if ((rc = set_active(c, mask_of(live)))) return rc;
    launch_winv(c->d_u, opt->RelTol, opt->AbsTol, c->d_winv, c->seg, s);
    launch_dot(c->d_g0, c->d_g0, c->seg, scal_slot(c, S_BETA2), HS, c->rw.partials, s);
    launch_dot(c->d_u, c->d_u, c->seg, scal_slot(c, S_NU2), HS, c->rw.partials, s);
    CK(cudaGetLastError());
    static_assert(S_NU2 == S_BETA2 + 1, "beta^2 and |u|^2 are fetched together");
    CK(cudaMemcpy2DAsync(c->h_stage, 2 * sizeof(double), scal_slot(c, S_BETA2), sizeof(double) * HS,
                         2 * sizeof(double), (size_t)S, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::vector<int> arn((size_t)S, 0);
    int narn = 0;
    for (int q : live) {
        ScenState& z = c->sc[q];
        std::fill(z.Hm.begin(), z.Hm.end(), 0.0);
        z.phi_m = 0;
        z.beta = std::sqrt(c->h_stage[2 * q]);
        z.nu = std::sqrt(c->h_stage[2 * q + 1]);
        z.eps = std::sqrt((1.0 + z.nu) * DBL_EPSILON);
        z.m = 0;
        z.happy = false;
        z.errK = 0.0;
        z.vnw = 0.0;
        z.iterating = z.beta != 0.0;
        c->h_eps[3 * q] = z.eps;
        c->h_eps[3 * q + 1] = 1.0 / z.eps;
        c->h_eps[3 * q + 2] = z.iterating ? 1.0 / z.beta : 0.0;
        if (z.iterating) {
            arn[q] = 1;
            ++narn;
        }
    }
    // Arnoldi, all iterating scenarios together
    if (narn > 0) {
        if ((rc = upload_eps(c))) return rc;
        if ((rc = set_active(c, arn))) return rc;
        launch_seg_scale(c->d_g0, scal_slot(c, S_IB), HS, V, c->seg, s);
        // The first batch of Arnoldi steps is launched back to back up to the
        // smallest Krylov dimension the iterating scenarios took last time;
        // their columns are then checked in order exactly as if each had been
        // read back alone (steps past a scenario's stopping point only write
        // columns it never uses).  Further steps go one at a time.
        int pred = c->maxk;
        for (int q = 0; q < S; ++q)
            if (arn[q]) pred = std::min(pred, std::max(1, c->sc[q].m_prev));
        int j = 0;
        while (j < c->maxk && narn > 0) {
            const int nb = (j == 0) ? std::max(1, std::min(pred, c->maxk)) : 1;
            if ((rc = set_active(c, arn))) return rc;
            const double frac = (double)narn / S;
            for (int jj = j; jj < j + nb; ++jj) {
                if (c->use_graphs) {
                    cudaGraphExec_t& ge = c->graphs[(size_t)jj];
                    std::array<cudaEvent_t, 4>& ev = c->graph_ev[(size_t)jj];
                    if (!ge) {
                        for (auto& e : ev)
                            if (!e) CK(cudaEventCreate(&e));
                        for (int attempt = 0; attempt < 2 && !ge; ++attempt) {
                            set_counting(false);
                            CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                            // event-record nodes only while profiling
                            arnoldi_kernels(c, jj, c->prof ? ev.data() : nullptr, frac);
                            cudaGraph_t g = nullptr;
                            cudaError_t ce = cudaStreamEndCapture(s, &g);
                            set_counting(true);
                            if (ce == cudaSuccess) ce = cudaGraphInstantiate(&ge, g, 0);
                            if (g) cudaGraphDestroy(g);
                            if (ce != cudaSuccess) {
                                // a cooperative launch that cannot be captured:
                                // capture the separate Gram-Schmidt kernels
                                ge = nullptr;
                                cudaGetLastError();
                                if (!c->fused_gs || attempt == 1 || c->gs_variant == 1) CK(ce);
                                c->fused_gs = false;
                                for (auto& x : c->graphs)
                                    if (x) {
                                        cudaGraphExecDestroy(x);
                                        x = nullptr;
                                    }
                            }
                        }
                    }
                    CK(cudaGraphLaunch(ge, s));
                    add_launches((c->fused_gs || c->gs_variant == 1) ? 3 : jj + 6);
                } else {
                    arnoldi_kernels(c, jj, nullptr, frac);
                }
            }
            CK(cudaGetLastError());
            // columns j..j+nb-1 of every H and the weighted norms of v_{j+1..j+nb}
            const size_t row = (size_t)nb * ldH + (size_t)nb;
            CK(cudaMemcpy2DAsync(c->h_stage, sizeof(double) * row, c->d_scal + (size_t)j * ldH,
                                 sizeof(double) * HS, sizeof(double) * (size_t)nb * ldH, (size_t)S,
                                 cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpy2DAsync(c->h_stage + (size_t)nb * ldH, sizeof(double) * row, scal_slot(c, S_COUNT + j),
                                 sizeof(double) * HS, sizeof(double) * (size_t)nb, (size_t)S,
                                 cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (c->fused_gs || c->gs_variant == 1) {
                int e = 0;
                CK(cudaMemcpy(&e, c->d_gserr, sizeof(int), cudaMemcpyDeviceToHost));
                if (e) {
                    set_error("Gram-Schmidt: a grid barrier wait expired");
                    cudaMemset(c->d_gserr, 0, sizeof(int));
                    cudaMemset(c->d_gsbar, 0, 2 * sizeof(unsigned int));   // a count left mid-barrier
                    return TSR_ERR_TIMEOUT;
                }
            }
            phi_batch(c, arn, j, nb, row, opt->MinKrylov, phi_jobs, phi_slot, phi_buf);
            for (int jj = j; jj < j + nb && narn > 0; ++jj) {
                if (c->use_graphs && c->prof) {
                    std::array<cudaEvent_t, 4>& ev = c->graph_ev[(size_t)jj];
                    float ta = 0.f, tb = 0.f;
                    CK(cudaEventElapsedTime(&ta, ev[0], ev[1]));
                    CK(cudaEventElapsedTime(&tb, ev[2], ev[3]));
                    c->prof_acc_ms[0] += ta;
                    c->prof_acc_bytes[0] += frac * g_bytes(c, true);
                    c->prof_acc_n[0] += 1;
                    c->prof_acc_ms[1] += tb;
                    c->prof_acc_bytes[1] += frac * 8.0 * (double)N * (double)(jj + 3);
                    c->prof_acc_n[1] += 1;
                }
                for (int q = 0; q < S; ++q) {
                    if (!arn[q]) continue;
                    ScenState& z = c->sc[q];
                    io.st[q].FuncEvals++;
                    const double* col = c->h_stage + (size_t)q * row + (size_t)(jj - j) * ldH;
                    double hs = 0.0;
                    for (int i = 0; i <= jj; ++i) {
                        z.Hm[(size_t)jj * ldH + i] = col[i];
                        hs = std::fma(col[i], col[i], hs);
                    }
                    const double hn = col[jj + 1];
                    z.Hm[(size_t)jj * ldH + jj + 1] = hn;
                    const double Sv = c->h_stage[(size_t)q * row + (size_t)nb * ldH + (size_t)(jj - j)];
                    z.m = jj + 1;
                    bool stop = false;
                    if (!(hn > 1e-12 * std::sqrt(std::fma(hn, hn, hs)))) {
                        z.happy = true;
                        stop = true;
                    } else if (!(z.m < opt->MinKrylov && z.m < z.maxk)) {
                        z.vnw = std::sqrt(Sv / (double)Ns(q));
                        // the batch's evaluation of phi_1(dt H_m) for this scenario and m
                        const int jb = phi_slot[(size_t)q * nb + (size_t)(jj - j)];
                        if (jb < 0) {
                            set_error("internal: phi_1 evaluation missing from the batch");
                            return TSR_ERR_ARG;
                        }
                        const PhiJob& J = phi_jobs[(size_t)jb];
                        rc = J.rc;
                        if (rc) {
                            set_error("phipade: singular Pade denominator");
                            z.phi_m = 0;
                        } else {
                            for (int cc = 0; cc < z.m; ++cc)
                                std::memcpy(z.phi.data() + (size_t)cc * c->maxk,
                                            phi_buf.data() + J.off + (size_t)cc * c->maxk, sizeof(double) * z.m);
                            z.phi_m = z.m;
                            z.phi_alpha = z.dt;
                        }
                        if (rc) {
                            fail(q, rc, "phipade: singular Pade denominator");
                            stop = true;
                        } else {
                            z.errK = std::fabs(((z.dt * z.beta) * hn) * z.phi[(size_t)z.m - 1]) * z.vnw;
                            if (z.errK <= kKrylovTol) stop = true;
                        }
                    }
                    if (z.m >= z.maxk) stop = true;
                    if (stop) {
                        arn[q] = 0;
                        --narn;
                    }
                }
            }
            j += nb;
        }
    }
    // Krylov error too large at the largest dimension: shorten the step
    for (int q : live) {
        ScenState& z = c->sc[q];
        if (z.status || z.beta == 0.0 || z.happy) continue;
        while (z.errK > kKrylovTol) {
            const double f = 0.5 > opt->MinStepDecFac ? 0.5 : opt->MinStepDecFac;
            z.dt = z.dt * f;
            z.diag_krylov_cuts++;
            z.last = false;
            if (z.dt < opt->MinStep) {
                fail(q, TSR_ERR_MINSTEP, "step size below MinStep (Krylov)");
                break;
            }
            if ((rc = phi_host(c, z, z.dt, z.m))) {
                fail(q, rc, "phipade: singular Pade denominator");
                break;
            }
            z.errK = std::fabs(((z.dt * z.beta) * z.Hm[(size_t)(z.m - 1) * ldH + z.m]) *
                               z.phi[(size_t)z.m - 1]) * z.vnw;
        }
    }
    // step attempts: u_new = u + dt beta V phi_1(dt H) e_1, G(u_new), error
    std::vector<int> pend;
    for (int q : live)
        if (!c->sc[q].status) pend.push_back(q);
    const int zoff = mk1 + 1, doff = c->CS - 1;
    std::vector<double> errs((size_t)S);
    while (!pend.empty()) {
        CK(cudaStreamSynchronize(s));   // staging buffers may still be in flight
        std::vector<int> go;
        for (int q : pend) {
            ScenState& z = c->sc[q];
            const int m = z.m;
            int mz = 0;
            if (m > 0) {
                // phi_1(dt H_m) from the Krylov tests when dt is still theirs
                if (!(z.phi_m == m && z.phi_alpha == z.dt) && (rc = phi_host(c, z, z.dt, m))) {
                    fail(q, rc, "phipade: singular Pade denominator");
                    continue;
                }
                const double dtb = z.dt * z.beta;
                for (int i = 0; i < m; ++i) z.cv[i] = dtb * z.phi[i];
                mz = z.happy ? m : m + 1;
                for (int i = 0; i < mz; ++i) {
                    double a = 0.0;
                    for (int k = 0; k < m; ++k) a = std::fma(z.Hm[(size_t)k * ldH + i], z.cv[k], a);
                    z.z[i] = a;
                }
            }
            double* cq = c->h_coef + (size_t)q * c->CS;
            for (int i = 0; i < m; ++i) cq[i] = z.cv[i];
            for (int i = 0; i < mz; ++i) cq[zoff + i] = z.z[i];
            cq[doff] = z.dt / 3.0;
            c->h_mint[q] = m;
            c->h_mint[S + q] = mz;
            go.push_back(q);
        }
        pend.swap(go);
        if (pend.empty()) break;
        if ((rc = set_active(c, mask_of(pend)))) return rc;
        CK(cudaMemcpyAsync(c->d_coef, c->h_coef, sizeof(double) * (size_t)c->CS * S, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(c->d_mint, c->h_mint, sizeof(int) * 2 * (size_t)S, cudaMemcpyHostToDevice, s));
        launch_combine(c->d_u, V, N, c->d_coef, c->CS, c->d_mint, c->d_unew, c->seg, s);
        if ((rc = reset_flag(c))) return rc;
        int pe = prof_begin(c, 0, g_bytes(c, false) * pend.size() / S);
        launch_g(c->P, 0, c->d_unew, nullptr, nullptr, nullptr, c->d_g1, s);
        prof_end(c, pe);
        for (int q : pend) io.st[q].FuncEvals++;
        launch_err(c->d_g1, c->d_g0, V, N, c->d_coef + zoff, c->CS, c->d_mint + S, c->d_coef + doff, c->CS,
                   c->d_winv, c->seg, scal_slot(c, S_ERR), HS, c->rw.partials, c->d_w, s);
        CK(cudaGetLastError());
        if ((rc = read_flags(c))) return rc;
        if ((rc = fetch_scalars(c, S_ERR, errs.data()))) return rc;
        std::vector<int> acc, next;
        for (int q : pend) {
            ScenState& z = c->sc[q];
            double err = 0.0;
            if (c->h_flag[q]) err = INFINITY;
            else if (z.m > 0) err = std::sqrt(errs[q] / (double)Ns(q));
            z.err = err;
            if (err <= 1.0) {
                acc.push_back(q);
                continue;
            }
            double fac = (err == err && err < INFINITY) ? opt->SafetyFac * std::pow(err, -1.0 / 3.0)
                                                         : opt->MinStepDecFac;
            if (fac < opt->MinStepDecFac) fac = opt->MinStepDecFac;
            if (fac > 1.0) fac = opt->MinStepDecFac;
            z.dt = z.dt * fac;
            z.last = false;
            z.diag_rejects++;
            if (z.dt < opt->MinStep) {
                fail(q, TSR_ERR_MINSTEP, "step size below MinStep");
                continue;
            }
            next.push_back(q);
        }
        // accepted: solutions at the tspan times inside the step, then the
        // new state and its G
        const int ns = (int)io.tspan[0];
        for (int q : acc) {
            ScenState& z = c->sc[q];
            const double tn = z.last ? io.tend : z.t + z.dt;
            double* rows = io.solns ? io.solns[q] : nullptr;
            if (!rows) continue;
            const long long off = c->scen_start[q], n = Ns(q);
            for (int k = 1; k <= ns; ++k) {
                if (!(io.tspan[k] > z.t && io.tspan[k] <= tn)) continue;
                double* row = rows + (size_t)k * (size_t)n;
                if (z.m == 0 && c->calibrated_output) {
                    CK(cudaMemcpyAsync(c->d_x, c->d_u, sizeof(double) * (size_t)N, cudaMemcpyDeviceToDevice, s));
                    launch_calibrate(c->P, c->d_x, s);
                    CK(cudaMemcpyAsync(row, c->d_x + off, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s));
                } else if (z.m == 0) {
                    CK(cudaMemcpyAsync(row, c->d_u + off, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s));
                } else {
                    const double tau = io.tspan[k] - z.t;
                    if ((rc = phi_host(c, z, tau, z.m))) {
                        fail(q, rc, "phipade: singular Pade denominator");
                        break;
                    }
                    const double tb = tau * z.beta;
                    CK(cudaStreamSynchronize(s));
                    double* cq = c->h_coef + (size_t)q * c->CS;
                    for (int i = 0; i < z.m; ++i) cq[i] = tb * z.phi[i];
                    CK(cudaMemcpyAsync(c->d_coef + (size_t)q * c->CS, cq, sizeof(double) * (size_t)z.m,
                                       cudaMemcpyHostToDevice, s));
                    if ((rc = set_active(c, mask_of({q})))) return rc;
                    launch_combine(c->d_u, V, N, c->d_coef, c->CS, c->d_mint, c->d_x, c->seg, s);
                    if (c->calibrated_output) launch_calibrate(c->P, c->d_x, s);
                    CK(cudaMemcpyAsync(row, c->d_x + off, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s));
                }
                CK(cudaStreamSynchronize(s));
            }
        }
        std::vector<int> ok;
        for (int q : acc)
            if (!c->sc[q].status) ok.push_back(q);
        if (!ok.empty()) {
            if ((rc = set_active(c, mask_of(ok)))) return rc;
            launch_seg_copy2(c->d_unew, c->d_u, c->d_g1, c->d_g0, c->seg, s);
            CK(cudaGetLastError());
        }
        for (int q : ok) {
            ScenState& z = c->sc[q];
            exprem_stats_struct& st = io.st[q];
            const double tn = z.last ? io.tend : z.t + z.dt;
            z.t = tn;
            double fac = (z.err > 0.0) ? opt->SafetyFac * std::pow(z.err, -1.0 / 3.0) : opt->MaxStepIncFac;
            z.diag_capped = fac >= opt->MaxStepIncFac;
            z.diag_err = z.err;
            if (fac > opt->MaxStepIncFac) fac = opt->MaxStepIncFac;
            if (fac < opt->MinStepDecFac) fac = opt->MinStepDecFac;
            double dn = z.dt * fac;
            if (dn > opt->MaxStep) dn = opt->MaxStep;
            if (dn < opt->MinStep) dn = opt->MinStep;
            st.CurrentStep = dn;
            st.CurrentTime = tn;
            st.CurrentKryDim = z.m;
            st.NumSteps++;
            z.g0_valid = true;
            z.m_prev = z.m;
        }
        pend.swap(next);
    }
    CK(cudaStreamSynchronize(s));
    return TSR_OK;
}

}  // namespace

extern "C" int tsr_exprem_advance(tsr_ctx* c, double tend, const double* tspan, double* tspan_solns,
                                  const exprem_options_struct* opt, exprem_stats_struct* st,
                                  double* t_out)
{
    if (!c || !opt || !st || !tspan || !c->sc[0].loaded) return TSR_ERR_ARG;
    if (c->S != 1) {
        set_error("a context of several scenarios advances with tsr_ensemble_advance");
        return TSR_ERR_ARG;
    }
    if (c->maxk < 1) {
        set_error("context created without a Krylov basis (max_krylov = 0)");
        return TSR_ERR_ARG;
    }
    double* solns[1] = {tspan_solns};
    RoundIO io{tend, tspan, solns, opt, st};
    int rc = exprem_round(c, std::vector<int>{0}, io);
    if (rc) return rc;
    if (c->sc[0].status) return c->sc[0].status;
    if (t_out) *t_out = c->sc[0].t;
    return TSR_OK;
}

extern "C" int tsr_ensemble_advance(tsr_ctx* c, double tend, const double* tspan, double* const* tspan_solns,
                                    const exprem_options_struct* opt, exprem_stats_struct* stats,
                                    double* t, int* status, int* n_running)
{
    if (!c || !opt || !stats || !tspan || !t || !status || !c->sc[0].loaded) return TSR_ERR_ARG;
    if (c->maxk < 1) {
        set_error("context created without a Krylov basis (max_krylov = 0)");
        return TSR_ERR_ARG;
    }
    std::vector<int> part;
    for (int q = 0; q < c->S; ++q)
        if (c->sc[q].status == TSR_OK && c->sc[q].t < tend) part.push_back(q);
    RoundIO io{tend, tspan, tspan_solns, opt, stats};
    int rc = part.empty() ? TSR_OK : exprem_round(c, part, io);
    int run = 0;
    for (int q = 0; q < c->S; ++q) {
        t[q] = c->sc[q].t;
        status[q] = c->sc[q].status;
        if (status[q] == TSR_OK && t[q] < tend) ++run;
    }
    if (n_running) *n_running = run;
    return rc;
}

extern "C" int tsr_exprem_step(tsr_ctx* c, double* t, double tend, const double* tspan,
                               double* tspan_solns, double* u0, const exprem_options_struct* opt,
                               exprem_stats_struct* st)
{
    if (!c || !t || !u0 || !opt || !st || !tspan) return TSR_ERR_ARG;
    // reuse G(u) of the previous accepted step when the caller hands back
    // the same state (same array, same time)
    ScenState& z = c->sc[0];
    const bool cached = z.loaded && z.g0_valid && c->last_u0 == u0 && c->last_t == *t && *t != 0.0;
    int rc;
    if (cached) {
        CK(cudaMemcpyAsync(c->d_u, u0, sizeof(double) * (size_t)c->N, cudaMemcpyHostToDevice,
                           c->stream));
        z.t = *t;
    } else {
        if ((rc = tsr_exprem_load(c, u0, *t))) return rc;
    }
    st->CurrentSoln = u0;
    double tn = *t;
    rc = tsr_exprem_advance(c, tend, tspan, tspan_solns, opt, st, &tn);
    if (rc != TSR_OK) return rc;
    if ((rc = tsr_exprem_store(c, u0))) return rc;
    *t = tn;
    c->last_u0 = u0;
    c->last_t = tn;
    return TSR_OK;
}

// ---- implicit contexts of the drop-in entry points ---------------------------
namespace {
std::mutex g_reg_mu;
std::map<const void*, tsr_ctx*> g_reg;
tsr_model_ext g_default_ext{};
bool g_have_ext = false;
int g_default_maxk = 100;
}  // namespace

namespace tsr {
tsr_ctx* registry_get(const user_data_struct* ud, int* rc)
{
    std::lock_guard<std::mutex> lk(g_reg_mu);
    const void* key = ud->macro_mesh.elements;
    auto it = g_reg.find(key);
    if (it != g_reg.end()) {
        *rc = TSR_OK;
        return it->second;
    }
    tsr_ctx* c = tsr_init(ud, g_have_ext ? &g_default_ext : nullptr, nullptr, g_default_maxk);
    if (!c) {
        *rc = TSR_ERR_CUDA;
        return nullptr;
    }
    g_reg[key] = c;
    *rc = TSR_OK;
    return c;
}
}  // namespace tsr

extern "C" int tsr_set_default_ext(const tsr_model_ext* ext, int max_krylov)
{
    std::lock_guard<std::mutex> lk(g_reg_mu);
    if (ext) {
        g_default_ext = *ext;
        g_have_ext = true;
    } else {
        g_have_ext = false;
    }
    if (max_krylov > 0) g_default_maxk = max_krylov;
    return TSR_OK;
}

extern "C" void tsr_release_all(void)
{
    std::lock_guard<std::mutex> lk(g_reg_mu);
    for (auto& kv : g_reg) tsr_free(kv.second);
    g_reg.clear();
}

extern "C" int tsr_gfunc_gpu(double* g, double* u, const user_data_struct* ud)
{
    if (!g || !u || !ud) return TSR_ERR_ARG;
    int rc;
    tsr_ctx* c = tsr::registry_get(ud, &rc);
    if (!c) return rc;
    return tsr_g_eval(c, u, g);
}

// ---- measurement hooks ----------------------------------------------------------

extern "C" int tsr_profile(tsr_ctx* c, int enable)
{
    if (!c) return TSR_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    if ((enable != 0) != c->prof) {
        // the Arnoldi graphs carry timing events only while profiling
        for (auto& g : c->graphs)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    }
    c->prof = enable != 0;
    c->prof_used = 0;
    for (int q = 0; q < 2; ++q) {
        c->prof_acc_ms[q] = 0.0;
        c->prof_acc_bytes[q] = 0.0;
        c->prof_acc_n[q] = 0;
    }
    return TSR_OK;
}

extern "C" int tsr_profile_read(tsr_ctx* c, int cat, double* ms, long long* count, double* bytes)
{
    if (!c || !ms || !count || !bytes) return TSR_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    double t = 0.0, b = 0.0;
    long long n = 0;
    for (size_t i = 0; i < c->prof_used; ++i) {
        const tsr_ctx::ProfEv& e = c->prof_ev[i];
        if (e.cat != cat) continue;
        float x = 0.f;
        CK(cudaEventElapsedTime(&x, e.a, e.b));
        t += x;
        b += e.bytes;
        ++n;
    }
    if (cat == 0 || cat == 1) {
        t += c->prof_acc_ms[cat];
        b += c->prof_acc_bytes[cat];
        n += c->prof_acc_n[cat];
    }
    *ms = t;
    *count = n;
    *bytes = b;
    return TSR_OK;
}

extern "C" unsigned long long tsr_kernel_launches(void) { return tsr::kernel_launches(); }

extern "C" int tsr_fp64_peak(double* ops_per_s)
{
    if (!ops_per_s) return TSR_ERR_ARG;
    if (tsr::measure_fp64_peak(ops_per_s)) {
        set_error("FP64 peak probe failed");
        return TSR_ERR_CUDA;
    }
    return TSR_OK;
}

extern "C" int tsr_mark(tsr_ctx* c, int slot)
{
    if (!c || slot < 0 || slot >= 16) return TSR_ERR_ARG;
    if (!c->marks[slot]) CK(cudaEventCreate(&c->marks[slot]));
    CK(cudaEventRecord(c->marks[slot], c->stream));
    return TSR_OK;
}

extern "C" int tsr_elapsed_ms(tsr_ctx* c, int a, int b, double* ms)
{
    if (!c || !ms || a < 0 || b < 0 || a >= 16 || b >= 16 || !c->marks[a] || !c->marks[b])
        return TSR_ERR_ARG;
    CK(cudaEventSynchronize(c->marks[b]));
    float x = 0.f;
    CK(cudaEventElapsedTime(&x, c->marks[a], c->marks[b]));
    *ms = x;
    return TSR_OK;
}

extern "C" int tsr_sync(tsr_ctx* c)
{
    if (!c) return TSR_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaDeviceSynchronize());
    return TSR_OK;
}

extern "C" void* tsr_pinned_alloc(size_t bytes)
{
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) {
        set_error("cudaMallocHost failed");
        return nullptr;
    }
    return p;
}

extern "C" void tsr_pinned_free(void* p)
{
    if (p) cudaFreeHost(p);
}

// ---- autotuner of the cell kernel's packing and block size ---------------------
// Times G on the given state for every (threads, shared-memory budget) pair
// that fits and keeps the fastest plan.  Plans differ only in how cells are
// packed into CTAs; every plan gives the same bits.

extern "C" int tsr_autotune(tsr_ctx* c, const double* u_host, int reps, double* best_ms,
                            int* best_threads, int* best_budget)
{
    if (!c || !u_host) return TSR_ERR_ARG;
    if (reps < 1) reps = 3;
    CK(cudaMemcpyAsync(c->d_x, u_host, sizeof(double) * (size_t)c->N, cudaMemcpyHostToDevice, c->stream));
    int rc0 = all_active(c);
    if (rc0) return rc0;
    // block sizes include warp counts that divide the node and element
    // counts of common templates evenly (the phases of a bundle wait for
    // their slowest warp)
    const int thr[] = {128, 160, 192, 224, 256, 288, 320, 384, 448, 512, 768, 1024};
    // budgets from one cell per bundle (0: every CTA takes a single cell, the
    // most CTAs for small problems, whose cells' long per-node chains then
    // run side by side) to large bundles
    const int bud[] = {0, 16 * 1024, 32 * 1024, 48 * 1024, 64 * 1024, 96 * 1024, 144 * 1024, 200 * 1024};
    double best = 1e30;
    int bt = c->tuned_threads, bb = c->tuned_budget;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    struct EventGuard {
        cudaEvent_t* a;
        cudaEvent_t* b;
        ~EventGuard()
        {
            if (*a) cudaEventDestroy(*a);
            if (*b) cudaEventDestroy(*b);
        }
    } guard{&e0, &e1};
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int bs = c->tuned_tables;
    for (int tab : {1, 0})
    for (int T : thr)
        for (int B : bud) {
            if (B > c->dev_smem) continue;
            if (tsr::plan_cells(c, T, B, tab) != TSR_OK) continue;
            launch_g(c->P, 0, c->d_x, nullptr, nullptr, nullptr, c->d_y, c->stream);   // warm
            CK(cudaEventRecord(e0, c->stream));
            for (int r = 0; r < reps; ++r)
                launch_g(c->P, 0, c->d_x, nullptr, nullptr, nullptr, c->d_y, c->stream);
            CK(cudaEventRecord(e1, c->stream));
            CK(cudaEventSynchronize(e1));
            CK(cudaGetLastError());
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (ms / reps < best) {
                best = ms / reps;
                bt = T;
                bb = B;
                bs = tab;
            }
        }
    int rc = tsr::plan_cells(c, bt, bb, bs);
    if (rc) return rc;
    if (best_ms) *best_ms = best;
    if (best_threads) *best_threads = bt;
    if (best_budget) *best_budget = bb;
    return TSR_OK;
}

extern "C" int tsr_set_cell_plan(tsr_ctx* c, int threads, int budget, int tables_smem)
{
    if (!c || threads < 64 || threads > 1024 || threads % 32 != 0 || budget < 0 || budget > c->dev_smem)
        return TSR_ERR_ARG;
    return tsr::plan_cells(c, threads, budget, tables_smem ? 1 : 0);
}

extern "C" int tsr_cell_plan(tsr_ctx* c, int* out)
{
    if (!c || !out) return TSR_ERR_ARG;
    out[0] = c->P.micro_block;
    out[1] = c->tuned_budget;
    out[2] = c->P.tables_smem;
    out[3] = c->P.m.maxc;
    out[4] = c->P.micro_grid;
    out[5] = (int)c->P.micro_smem;
    return TSR_OK;
}

extern "C" int tsr_set_graphs(tsr_ctx* c, int enable)
{
    if (!c) return TSR_ERR_ARG;
    c->use_graphs = enable != 0;
    return TSR_OK;
}

extern "C" int tsr_step_diagnostics(tsr_ctx* c, int s, double* out)
{
    if (!c || !out || s < 0 || s >= c->S) return TSR_ERR_ARG;
    const ScenState& z = c->sc[s];
    out[0] = z.diag_dt0;
    out[1] = z.dt;
    out[2] = z.diag_err;
    out[3] = z.diag_krylov_cuts;
    out[4] = z.diag_rejects;
    out[5] = z.diag_capped;
    out[6] = z.m;
    out[7] = z.diag_clipped;
    return TSR_OK;
}

extern "C" int tsr_set_calibrated_output(tsr_ctx* c, int enable)
{
    if (!c) return TSR_ERR_ARG;
    c->calibrated_output = enable != 0;
    return TSR_OK;
}

extern "C" int tsr_calibrate_device(tsr_ctx* c, double* d_x)
{
    if (!c || !d_x) return TSR_ERR_ARG;
    int rc = all_active(c);
    if (rc) return rc;
    launch_calibrate(c->P, d_x, c->stream);
    CK(cudaGetLastError());
    return TSR_OK;
}

extern "C" int tsr_set_gram_schmidt(tsr_ctx* c, int variant)
{
    if (!c || variant < 0 || variant > 1) return TSR_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    if (variant == 1) {
        if (c->maxk > gs_cgs2_max_dim()) {
            set_error("tsr_set_gram_schmidt: classical Gram-Schmidt twice takes Krylov dimensions up to 63");
            return TSR_ERR_ARG;
        }
        if (c->gs2_grid < 1) c->gs2_grid = gs_cgs2_grid(c->nsm, c->maxk);
        if (c->gs2_grid < 1) {
            set_error("tsr_set_gram_schmidt: the CGS2 kernel cannot be launched on this device");
            return TSR_ERR_CUDA;
        }
        if (!c->d_gs2part) {
            void* p = nullptr;
            int rc = dev_alloc(c, sizeof(double) * 2 * (size_t)(c->maxk + 1) * (size_t)c->pstride, &p);
            if (rc) return rc;
            c->d_gs2part = (double*)p;
        }
    }
    c->gs_variant = variant;
    for (auto& g : c->graphs)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    return TSR_OK;
}

extern "C" int tsr_set_fused_gs(tsr_ctx* c, int enable)
{
    if (!c || enable < 0 || enable > 2) return TSR_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    c->fused_gs = enable != 0 && c->gs_grid > 0;
    c->gs_small_warps = enable == 2 ? 0 : 1;
    for (auto& g : c->graphs)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    return TSR_OK;
}

// ---- learned closure ------------------------------------------------------------
// Cells switch between the micro mesh (plain FP64 cell kernel) and the
// learned closure between steps; the unknown vector is re-laid out on the
// device and the Arnoldi graphs are captured again.

namespace {

int relayout(tsr_ctx* c, const std::vector<int>& learned_new)
{
    const int Ne = c->Ne, Mn = c->Mn;
    Problem& P = c->P;
    cudaStream_t s = c->stream;
    // interior mean water content of the cells that become learned
    launch_cell_summary(P, c->d_u, nullptr, nullptr, c->d_summary, s);
    std::vector<long long> off((size_t)Ne);
    long long N = Mn;
    std::vector<int> lc;
    for (int k = 0; k < Ne; ++k) {
        off[k] = N;
        N += learned_new[k] ? 1 : c->tpl_nodes[c->tpl_full_host[k]];
        c->cell_tpl_host[k] = learned_new[k] ? c->pseudo_tpl : c->tpl_full_host[k];
        if (learned_new[k]) lc.push_back(k);
    }
    const int nb = 1 - c->cur;
    CK(cudaStreamSynchronize(s));
    CK(cudaMemcpyAsync(c->d_off[nb], off.data(), sizeof(long long) * (size_t)Ne, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(c->d_learned[nb], learned_new.data(), sizeof(int) * (size_t)Ne, cudaMemcpyHostToDevice, s));
    launch_relayout(P, Mn, Ne, c->d_off[c->cur], c->d_learned[c->cur], c->d_off[nb], c->d_learned[nb],
                    c->d_summary, c->d_u, c->d_unew, s);
    CK(cudaGetLastError());
    // cells that become learned start a new head history
    std::vector<int> fresh;
    for (int k = 0; k < Ne; ++k)
        if (learned_new[k] && !c->learned_host[k]) fresh.push_back(k);
    CK(cudaMemcpyAsync(c->d_cell_tpl, c->cell_tpl_host.data(), sizeof(int) * (size_t)Ne, cudaMemcpyHostToDevice, s));
    if (!lc.empty())
        CK(cudaMemcpyAsync(c->d_lcells, lc.data(), sizeof(int) * lc.size(), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    if (!fresh.empty()) {
        std::vector<int> hc((size_t)Ne);
        CK(cudaMemcpy(hc.data(), c->d_hcount, sizeof(int) * (size_t)Ne, cudaMemcpyDeviceToHost));
        for (int k : fresh) hc[k] = 0;
        CK(cudaMemcpy(c->d_hcount, hc.data(), sizeof(int) * (size_t)Ne, cudaMemcpyHostToDevice));
    }
    std::swap(c->d_u, c->d_unew);
    c->cur = nb;
    c->learned_host = learned_new;
    c->nl = (int)lc.size();
    P.m.cell_off = c->d_off[nb];
    c->N = N;
    P.N = N;
    c->scen_start[1] = N;
    int rc;
    if ((rc = make_seg(c, c->scen_start, &c->seg))) return rc;
    c->sc[0].g0_valid = false;
    return tsr::plan_cells(c, c->tuned_threads, c->tuned_budget, c->tuned_tables);
}

ClosureDev closure_dev(tsr_ctx* c)
{
    ClosureDev C = c->cdev;
    C.w = mlp_device_weights(c->mlp);
    C.p = mlp_device_params(c->mlp);
    C.w2 = c->mlp2 ? mlp_device_weights(c->mlp2) : nullptr;
    C.p2 = c->mlp2 ? mlp_device_params(c->mlp2) : nullptr;
    C.cells = c->d_lcells;
    C.n = c->nl;
    C.hist = c->d_hist;
    C.hcount = c->d_hcount;
    C.hcur = c->d_hcur;
    C.t[0] = c->sc[0].t;
    C.t[1] = c->thist[0];
    C.t[2] = c->thist[1];
    C.t[3] = c->thist[2];
    C.kappa = c->d_kappa;
    C.aint = c->d_aint;
    C.flags = c->d_flags;
    C.nflag = c->d_nflag;
    return C;
}

}  // namespace

extern "C" int tsr_closure_set_learned(tsr_ctx* c, const int* learned)
{
    if (!c || !learned) return TSR_ERR_ARG;
    if (!c->closure) {
        set_error("context built without the learned closure (tsr_model_ext.cell_learned)");
        return TSR_ERR_ARG;
    }
    std::vector<int> l((size_t)c->Ne);
    for (int k = 0; k < c->Ne; ++k) l[k] = learned[k] ? 1 : 0;
    return relayout(c, l);
}

extern "C" int tsr_closure_set_coef(tsr_ctx* c, const double* kappa)
{
    if (!c || !kappa || !c->closure) return TSR_ERR_ARG;
    CK(cudaMemcpyAsync(c->d_kappa, kappa, sizeof(double) * 2 * (size_t)c->Ne, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (auto& z : c->sc) z.g0_valid = false;
    return TSR_OK;
}

extern "C" int tsr_closure_read(tsr_ctx* c, int* learned, double* kappa, int* flags)
{
    if (!c || !c->closure) return TSR_ERR_ARG;
    const size_t Ne = (size_t)c->Ne;
    if (learned) std::memcpy(learned, c->learned_host.data(), sizeof(int) * Ne);
    if (kappa) CK(cudaMemcpyAsync(kappa, c->d_kappa, sizeof(double) * 2 * Ne, cudaMemcpyDeviceToHost, c->stream));
    if (flags) CK(cudaMemcpyAsync(flags, c->d_flags, sizeof(int) * Ne, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return TSR_OK;
}

extern "C" int tsr_closure_attach(tsr_ctx* c, tsr_mlp* mlp, const double* norm, const float* zrange, double thr,
                                  double qfloor, int auto_fallback)
{
    if (!c || !mlp || !norm || !zrange || !c->closure) return TSR_ERR_ARG;
    c->mlp = mlp;
    ClosureDev& C = c->cdev;
    for (int i = 0; i < 6; ++i) {
        C.fmu[i] = norm[i];
        C.fsd[i] = norm[6 + i];
        C.zlo[i] = zrange[i];
        C.zhi[i] = zrange[6 + i];
    }
    C.ymu[0] = norm[12];
    C.ymu[1] = norm[13];
    C.ysd[0] = norm[14];
    C.ysd[1] = norm[15];
    C.thr = thr;
    C.qfloor = qfloor;
    c->auto_fallback = auto_fallback != 0;
    return TSR_OK;
}

extern "C" int tsr_closure_attach_ensemble(tsr_ctx* c, tsr_mlp* second, double thr_ens)
{
    if (!c || !c->closure || (second && !(thr_ens > 0.0))) return TSR_ERR_ARG;
    c->mlp2 = second;
    c->cdev.thr_ens = thr_ens;
    return TSR_OK;
}

// Coefficients of the learned cells at the current state, and the
// indicator; returns the number of flagged cells in *n_flagged.
extern "C" int tsr_closure_update(tsr_ctx* c, int* n_flagged)
{
    if (!c || !c->closure || !c->mlp || !c->sc[0].loaded) return TSR_ERR_ARG;
    int rc0 = all_active(c);     // refuses an unusable context
    if (rc0) return rc0;
    // word 0: flagged cells; word 1: a bounded wait of the network expired
    CK(cudaMemsetAsync(c->d_nflag, 0, 2 * sizeof(int), c->stream));
    ClosureDev C = closure_dev(c);
    launch_closure_update(c->P, c->d_u, C, c->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    int w[2] = {0, 0};
    CK(cudaMemcpy(w, c->d_nflag, 2 * sizeof(int), cudaMemcpyDeviceToHost));
    if (w[1]) {
        c->unusable = true;
        set_error("closure update: a wait on the tensor-core barrier expired (context now unusable)");
        return TSR_ERR_TIMEOUT;
    }
    if (n_flagged) *n_flagged = w[0];
    c->sc[0].g0_valid = false;      // G changed with the coefficients
    return TSR_OK;
}

// One accepted step of the two-scale system with the learned closure:
// coefficients and indicator at the current state, fallback of the flagged
// cells to their micro meshes (when enabled), one EXPREM step, head history.
extern "C" int tsr_closure_advance(tsr_ctx* c, double tend, const double* tspan, double* tspan_solns,
                                   const exprem_options_struct* opt, exprem_stats_struct* st, double* t_out,
                                   int* n_fallback)
{
    if (!c || !opt || !st || !tspan || !c->closure || !c->sc[0].loaded) return TSR_ERR_ARG;
    int rc, nf = 0;
    const bool use = c->mlp && c->nl > 0;
    if (use) {
        if ((rc = tsr_closure_update(c, &nf))) return rc;
        // new coefficients change G: the G(u) kept from the last step is stale
        c->sc[0].g0_valid = false;
        if (nf > 0 && c->auto_fallback) {
            std::vector<int> flags((size_t)c->Ne);
            CK(cudaMemcpy(flags.data(), c->d_flags, sizeof(int) * (size_t)c->Ne, cudaMemcpyDeviceToHost));
            std::vector<int> l = c->learned_host;
            for (int k = 0; k < c->Ne; ++k)
                if (l[k] && flags[k]) l[k] = 0;
            if ((rc = relayout(c, l))) return rc;
        }
    }
    const double t0 = c->sc[0].t;
    if ((rc = tsr_exprem_advance(c, tend, tspan, tspan_solns, opt, st, t_out))) return rc;
    if (use && c->nl > 0) {
        launch_closure_push(closure_dev(c), c->stream);
        CK(cudaGetLastError());
        c->thist[2] = c->thist[1];
        c->thist[1] = c->thist[0];
        c->thist[0] = t0;
    }
    if (n_fallback) *n_fallback = nf;
    return TSR_OK;
}

// Per-cell summary of state u (host, current layout; NULL: the loaded
// state): 5 doubles per cell, H_c, theta, d theta/dt, Q, h(theta).
extern "C" int tsr_cell_summary(tsr_ctx* c, const double* u, double* out)
{
    if (!c || !out || c->S != 1) return TSR_ERR_ARG;
    int rc;
    if ((rc = all_active(c))) return rc;
    const double* du = c->d_u;
    if (u) {
        CK(cudaMemcpyAsync(c->d_x, u, sizeof(double) * (size_t)c->N, cudaMemcpyHostToDevice, c->stream));
        du = c->d_x;
    }
    c->P.qlog = c->d_qlog;
    launch_g(c->P, 0, du, nullptr, nullptr, nullptr, c->d_y, c->stream);
    c->P.qlog = nullptr;
    launch_cell_summary(c->P, du, c->d_y, c->d_qlog, c->d_summary, c->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, c->d_summary, sizeof(double) * 5 * (size_t)c->Ne, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return TSR_OK;
}

// ---- checkpoint / resume -------------------------------------------------------
// File layout (native byte order): "TSRCKPT1", int32 S, int64 N, then per
// scenario t, status, m_prev and the exprem_stats fields (CurrentStep,
// CurrentTime, CurrentKryDim, NumSteps, FuncEvals), then u (N doubles).
// G(u) is not stored: the first step after a resume evaluates it again.

namespace {
struct CkptScen {
    double t;
    int32_t status, m_prev;
    double cur_step, cur_time;
    int32_t kry_dim, num_steps, func_evals, pad;
};
const char kCkptMagic[8] = {'T', 'S', 'R', 'C', 'K', 'P', 'T', '1'};
}  // namespace

extern "C" int tsr_checkpoint_save(tsr_ctx* c, const char* path, const exprem_stats_struct* stats)
{
    if (!c || !path || !stats || !c->sc[0].loaded) return TSR_ERR_ARG;
    if (c->closure) {
        set_error("checkpoints of learned-closure contexts are not supported");
        return TSR_ERR_ARG;
    }
    std::vector<double> u((size_t)c->N);
    CK(cudaMemcpyAsync(u.data(), c->d_u, sizeof(double) * u.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        set_error(std::string("cannot open ") + path);
        return TSR_ERR_IO;
    }
    const int32_t S = c->S;
    const int64_t N = c->N;
    bool ok = std::fwrite(kCkptMagic, 1, 8, f) == 8 && std::fwrite(&S, sizeof S, 1, f) == 1 &&
              std::fwrite(&N, sizeof N, 1, f) == 1;
    for (int q = 0; q < c->S && ok; ++q) {
        CkptScen r{};
        r.t = c->sc[q].t;
        r.status = c->sc[q].status;
        r.m_prev = c->sc[q].m_prev;
        r.cur_step = stats[q].CurrentStep;
        r.cur_time = stats[q].CurrentTime;
        r.kry_dim = stats[q].CurrentKryDim;
        r.num_steps = stats[q].NumSteps;
        r.func_evals = stats[q].FuncEvals;
        ok = std::fwrite(&r, sizeof r, 1, f) == 1;
    }
    ok = ok && std::fwrite(u.data(), sizeof(double), u.size(), f) == u.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) {
        set_error(std::string("write failed: ") + path);
        return TSR_ERR_IO;
    }
    return TSR_OK;
}

extern "C" int tsr_checkpoint_load(tsr_ctx* c, const char* path, exprem_stats_struct* stats)
{
    if (!c || !path || !stats) return TSR_ERR_ARG;
    if (c->closure) {
        // the closure's head history, coefficients and cell layout are not
        // in the file, so a resumed closure run would not match its state
        set_error("checkpoints of learned-closure contexts are not supported");
        return TSR_ERR_ARG;
    }
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        set_error(std::string("cannot open ") + path);
        return TSR_ERR_IO;
    }
    char magic[8];
    int32_t S = 0;
    int64_t N = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kCkptMagic, 8) == 0 &&
              std::fread(&S, sizeof S, 1, f) == 1 && std::fread(&N, sizeof N, 1, f) == 1;
    if (!ok || S != c->S || N != c->N) {
        std::fclose(f);
        set_error("checkpoint does not match this context (format, scenarios or unknowns)");
        return TSR_ERR_ARG;
    }
    std::vector<CkptScen> rs((size_t)S);
    std::vector<double> u((size_t)N);
    ok = std::fread(rs.data(), sizeof(CkptScen), rs.size(), f) == rs.size() &&
         std::fread(u.data(), sizeof(double), u.size(), f) == u.size();
    std::fclose(f);
    if (!ok) {
        set_error(std::string("truncated checkpoint: ") + path);
        return TSR_ERR_IO;
    }
    CK(cudaMemcpyAsync(c->d_u, u.data(), sizeof(double) * u.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int q = 0; q < S; ++q) {
        ScenState& z = c->sc[q];
        z.loaded = true;
        z.t = rs[q].t;
        z.status = rs[q].status;
        z.m_prev = rs[q].m_prev;
        z.g0_valid = false;
        stats[q].CurrentStep = rs[q].cur_step;
        stats[q].CurrentTime = rs[q].cur_time;
        stats[q].CurrentKryDim = rs[q].kry_dim;
        stats[q].NumSteps = rs[q].num_steps;
        stats[q].FuncEvals = rs[q].func_evals;
    }
    c->last_u0 = nullptr;
    return TSR_OK;
}
