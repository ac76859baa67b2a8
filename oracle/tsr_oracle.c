/*
 * tsr_oracle.c -- CPU FP64 oracle of the two-scale Richards hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the library links, loads or calls
 * this file; the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it to check (and to time beside) the CUDA path.
 *
 * What it restates.  The reference's right-hand side and integrator bodies
 * are not in its source tree: compile.sh:18-21 names exprem.cpp,
 * Gfunc_serial.cpp and Gfunc_parallel.cpp, and none of them ships.  Their
 * interfaces do ship, and this file follows them:
 *   oracle_g          int Gfunc_serial(double* g, double* u, user_data_struct)
 *                     (include/main.h:21); with nthreads > 1 the OpenMP form
 *                     Gfunc_parallel (include/main.h:22, include/Gfunc_parallel.h,
 *                     thread count from user_data.NUM_THREADS, include/user_data.h:9)
 *   oracle_exprem_step  int exprem(...) (include/main.h:29-32), one accepted
 *                     step per call as the driver loop expects (src/main.cpp:313-341),
 *                     options src/set_exprem_options.cpp:16-26, helpers
 *                     weighted_norm / check_step / check_flag_Gfunc (include/exprem.h:27-30)
 *   oracle_phipade    int phipade(...) (src/phipade.cpp:15-216)
 * The model (two-scale Richards, model_type 3, src/main.cpp:187-192) and the
 * method (Jacobian-free exponential Rosenbrock-Euler with Arnoldi) are stated
 * from the mathematics; the choices the missing sources leave open are fixed
 * here, in comments at each step.
 *
 * Parity pinning.  phipade and the mesh preprocessing are pinned against the
 * reference's own src/phipade.cpp, src/macro_mesh_properties.cpp and
 * src/micro_mesh_properties.cpp compiled from the reference tree
 * (oracle/Makefile, target ref).  G, Jv and EXPREM have no reference body to
 * run: for them parity is unpinned by reference code and rests on the
 * physics checks in the tests (hydrostatic equilibrium, water balance,
 * symmetry, Jv consistency, mesh convergence).
 *
 * Arithmetic contract.  Compiled without contraction (-ffp-contract=off);
 * every fused multiply-add is an explicit fma().  Elementary functions come
 * from tsr_math.h (table-driven, the same bits on host and device).  The
 * summation order of every sum is fixed and written out below, so that a
 * device implementation that follows the same order reproduces G, Jv, the
 * Krylov basis and whole trajectories bit for bit.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/tsr_types.h"
#include "../twoscalerich_gb300/csrc/tsr_math.h"

static const tsr_math_tables T = TSR_MATH_TABLES_INIT;

#ifdef TSR_ORACLE_LIBM
/* CPU-native variant used only to time the CPU baseline: the same
 * algorithm with the host C library's log/exp/log1p/expm1 (what a CPU
 * implementation of Gfunc_parallel would call); its results differ from the
 * bitwise oracle in the last bits. */
#define tsr_log(x, t) log(x)
#define tsr_exp(x, t) exp(x)
#define tsr_expm1(x, t) expm1(x)
#define tsr_log1p_s(x, s, t) log1p(x)
#define tsr_log1p_unit(x, s1p, t) (*(s1p) = 1.0 + (x), log1p(x))
#endif

/* ------------------------------------------------------------------ */
/* Van Genuchten-Mualem relations (parameters include/soil.h:1-7; m = 1-1/n
 * as set at src/main.cpp:127,140).  For h < 0, with a = alpha|h|,
 * t = a^n, Se = (1+t)^-m:
 *   K(h) = Ks Se^(1/2) (1 - (1 - Se^(1/m))^m)^2,  1 - Se^(1/m) = t/(1+t)
 *   theta(h) = theta_r + (theta_s - theta_r) Se
 *   C(h) = dtheta/dh = (theta_s-theta_r) m n t Se / (|h| (1+t))
 *        = (theta_s-theta_r) m n Se / (|h| (1 + 1/t))
 * For h >= 0: K = Ks, theta = theta_s, C = 0.  A specific storage S_s is
 * added to C everywhere.  C is carried as the ratio Cn/Cd.                 */

typedef struct {
    double Ks, thr, ths, alpha, n, m;
    double dth, coefC, mh;
} vgpar;

static vgpar make_vgpar(const soil_struct* s)
{
    vgpar p;
    p.Ks = s->Ksat;
    p.thr = s->thetar;
    p.ths = s->thetas;
    p.alpha = s->alpha;
    p.n = s->n;
    p.m = s->m;
    p.dth = s->thetas - s->thetar;
    p.coefC = (p.dth * s->m) * s->n;
    p.mh = -0.5 * s->m;
    return p;
}

/* K, Cn, Cd and Se at head h.  With e = exp(-|n log(alpha|h|)|) = min(t, 1/t):
 *   t < 1:  log(1+t) = log1p(e),          log(t/(1+t)) = nL - log1p(e)
 *   t >= 1: log(1+t) = nL + log1p(e),     log(t/(1+t)) = -log1p(e)
 * so no difference of nearly equal logarithms is ever formed (dry soil,
 * t >> 1, would otherwise cancel), and t/(1+t) = e/(1+e) or 1/(1+e). */
static void vg_eval(double h, const vgpar* p, double* K, double* Cn, double* Cd, double* Se_out)
{
    /* sign tests and sign flips on the bits (equal to h < 0, -h, -|nL| and
     * nL >= 0 for every non-NaN value) */
    if (tsr_lt0(h)) {
        double ah = tsr_negate(h);
        double a = p->alpha * ah;
        double L = tsr_log(a, &T);
        double nL = p->n * L;
        double e = tsr_exp(tsr_negabs(nL), &T);
        double s1;
        double lp = tsr_log1p_unit(e, &s1, &T);
        int dry = tsr_ge0(nL);
        double l1 = dry ? nL + lp : lp;                /* log(1+t) */
        double y = dry ? -(p->m * lp) : p->m * (nL - lp);
        double X = tsr_exp(p->mh * l1, &T);           /* Se^(1/2) */
        double Se = X * X;
        double B = -tsr_expm1(y, &T);                  /* 1 - (t/(1+t))^m */
        *K = (p->Ks * X) * (B * B);
        *Cn = dry ? p->coefC * Se : p->coefC * (e * Se);
        *Cd = ah * s1;
        *Se_out = Se;
    } else {
        *K = p->Ks;
        *Cn = 0.0;
        *Cd = 1.0;
        *Se_out = 1.0;
    }
}

/* Head of material p at water content theta (inverse of the retention
 * curve): Se = (theta - thr) / dth, h = -((Se^(-1/m) - 1)^(1/n)) / alpha,
 * 0 at or above saturation, Se floored at 1e-12. */
static double vg_head(double theta, const vgpar* p)
{
    double Se = (theta - p->thr) / p->dth;
    if (!(Se < 1.0)) return 0.0;
    if (!(Se > 1e-12)) Se = 1e-12;
    double L = tsr_log(Se, &T);
    double tt = tsr_expm1(-(L / p->m), &T);
    double lt = tsr_log(tt, &T);
    return -(tsr_exp(lt / p->n, &T) / p->alpha);
}

/* ------------------------------------------------------------------ */
/* Effective conductivity Keff(h) (include/Keff.h:1-8; table layout of
 * src/read_effective_conductivity.cpp:52-56): linear interpolation in
 * log10|h| on the uniform grid logh_first + i*logr, clamped to the ends.   */

typedef struct {
    int n;
    double first, inv_logr;
    const double* Kv;
} keffpar;

static void keff_eval(double H, const keffpar* kp, double K[4])
{
    int n = kp->n;
    if (n < 2) {
        for (int c = 0; c < 4; ++c) K[c] = kp->Kv[c * n];
        return;
    }
    double x = tsr_log(fabs(H), &T) * TSR_INV_LN10;
    double pos = (x - kp->first) * kp->inv_logr;
    int i;
    double w;
    if (!(pos > 0.0)) {
        i = 0;
        w = 0.0;
    } else if (pos >= (double)(n - 1)) {
        i = n - 2;
        w = 1.0;
    } else {
        i = (int)pos;
        w = pos - (double)i;
    }
    for (int c = 0; c < 4; ++c) {
        double k0 = kp->Kv[c * n + i], k1 = kp->Kv[c * n + i + 1];
        K[c] = fma(w, k1 - k0, k0);
    }
}

/* ------------------------------------------------------------------ */
/* Fixed-order sums.
 * canon32: item i goes to lane i mod 32 (lane sums in ascending i, starting
 * from 0.0), then the 32 lane sums are combined by the butterfly
 * p[l] <- p[l] + p[l xor d] for d = 16, 8, 4, 2, 1; the result is p[0].
 * chunked vector reductions: block b of 8192 items, thread t of 256 sums
 * items b*8192 + s*256 + t for s = 0..31 in ascending s; each warp of 32
 * threads is combined by the butterfly; the 8 warp sums as
 * ((w0+w1)+(w2+w3))+((w4+w5)+(w6+w7)); the block sums P[b] are then
 * reduced by one block the same way, thread t summing P[t], P[t+256], ...  */

static double butterfly32(double* p)
{
    double q[32];
    for (int d = 16; d >= 1; d >>= 1) {
        for (int l = 0; l < 32; ++l) q[l] = p[l] + p[l ^ d];
        memcpy(p, q, sizeof q);
    }
    return p[0];
}

static double block256(double* acc)
{
    double w[8];
    for (int k = 0; k < 8; ++k) w[k] = butterfly32(acc + 32 * k);
    return ((w[0] + w[1]) + (w[2] + w[3])) + ((w[4] + w[5]) + (w[6] + w[7]));
}

#define CHUNK 8192
#define BLK 256

/* Threads of the vector passes and of the chunk loop of the reductions
 * (set from the nthreads argument of the EXPREM step).  Each chunk's
 * partial is formed by one thread in the fixed order above and the chunk
 * partials are combined in the fixed order, so the thread count changes
 * the speed, never the bits. */
static int o_threads = 1;

typedef double (*term_fn)(long i, const void* ctx, double acc);

static double chunked_reduce(long n, term_fn fn, const void* ctx)
{
    long nb = (n + CHUNK - 1) / CHUNK;
    if (nb == 0) return 0.0;
    double* P = (double*)malloc(sizeof(double) * (size_t)nb);
#pragma omp parallel for num_threads(o_threads) schedule(static) if (nb >= 64 && o_threads > 1)
    for (long b = 0; b < nb; ++b) {
        double acc[BLK];
        for (int t = 0; t < BLK; ++t) {
            double a = 0.0;
            for (int s = 0; s < CHUNK / BLK; ++s) {
                long i = b * CHUNK + (long)s * BLK + t;
                if (i < n) a = fn(i, ctx, a);
            }
            acc[t] = a;
        }
        P[b] = block256(acc);
    }
    double acc[BLK];
    for (int t = 0; t < BLK; ++t) {
        double a = 0.0;
        for (long i = t; i < nb; i += BLK) a = a + P[i];
        acc[t] = a;
    }
    double r = block256(acc);
    free(P);
    return r;
}

typedef struct { const double *x, *y, *z; double s; } vctx;

static double t_dot(long i, const void* c, double acc)
{
    const vctx* v = (const vctx*)c;
    return fma(v->x[i], v->y[i], acc);
}
static double t_sum(long i, const void* c, double acc)
{
    const vctx* v = (const vctx*)c;
    return acc + v->x[i];
}
/* (x_i * y_i)^2 where y holds the inverse error weights */
static double t_wsq(long i, const void* c, double acc)
{
    const vctx* v = (const vctx*)c;
    double r = v->x[i] * v->y[i];
    return fma(r, r, acc);
}

double oracle_dot(const double* x, const double* y, long n)
{
    vctx c = {x, y, 0, 0};
    return chunked_reduce(n, t_dot, &c);
}

double oracle_vsum(const double* x, long n)
{
    vctx c = {x, 0, 0, 0};
    return chunked_reduce(n, t_sum, &c);
}

double oracle_wsq(const double* x, const double* winv, long n)
{
    vctx c = {x, winv, 0, 0};
    return chunked_reduce(n, t_wsq, &c);
}

/* ------------------------------------------------------------------ */
/* Problem handle                                                       */

typedef struct oracle_problem {
    user_data_struct ud;
    vgpar pA, pB;
    keffpar kp;
    double epsA, inv_Y, Ss, hD;
    int kface;
    const double* cell_scale;
    unsigned char* dirichlet;   /* [Mn] */
    /* micro templates: one (user_data.micro_mesh) or, in the batched form,
     * tsr_model_ext.templates with a template per cell */
    int ntpl;
    const micro_mesh_struct* tpl;       /* [ntpl] */
    double** faceH;             /* [ntpl][6*mNe]: per SCV face j of element e, D1/2, D2/2 */
    const int* cell_tpl;        /* [Ne] or NULL (all template 0) */
    long* cell_off;             /* [Ne] first unknown of cell k */
    vgpar* cell_pB;             /* [Ne] or NULL (all pB) */
    int max_mn, max_mNe;
    /* ensemble form: S scenarios, scenario-major unknowns */
    int S, scen_nodes, scen_cells;
    long* node_off;             /* [Mn] unknown index of macro node i */
    long* scen_start;           /* [S+1] */
    vgpar* scen_pA;             /* [S] or NULL (all pA) */
    double* scen_kscale;        /* [S] or NULL (all 1) */
    /* learned closure: cells with learned[k] carry one unknown */
    const int* learned;         /* [Ne] or NULL */
    const double* kappa;        /* [2 Ne] or NULL */
    long N;
    int Mn, Ne, nv, mn, mNe;
    /* EXPREM workspace */
    int maxk;
    double *V, *Hm, *phi, *g0, *g1, *w, *unew, *winv, *x, *D, *Dt;
    /* cached G(u) of the last accepted state */
    const double* cache_u;
    double cache_t;
    int cache_valid;
    /* Gram-Schmidt of the Arnoldi step: 0 modified (MGS), 1 classical
     * twice (CGS2) */
    int gs_variant;
} oracle_problem;

oracle_problem* oracle_create(const user_data_struct* ud, const tsr_model_ext* ext)
{
    if (!ud) return NULL;
    if (!(ext && ext->n_templates > 0) && ud->micro_mesh.no_verts != 3) return NULL;
    oracle_problem* P = (oracle_problem*)calloc(1, sizeof(oracle_problem));
    P->ud = *ud;
    P->pA = make_vgpar(&ud->soilA);
    P->pB = make_vgpar(&ud->soilB);
    P->kp.n = ud->effective_conductivity.no_hvalues;
    P->kp.first = ud->effective_conductivity.logh_first;
    P->kp.inv_logr = 1.0 / ud->effective_conductivity.logr;
    P->kp.Kv = ud->effective_conductivity.Keff_values;
    P->epsA = ud->effective_conductivity.epsilonA;
    P->Ss = (ext && ext->specific_storage > 0.0) ? ext->specific_storage : 1e-6;
    P->hD = ext ? ext->dirichlet_h : 0.0;
    P->kface = ext ? ext->kface_mode : 0;
    P->cell_scale = ext ? ext->cell_scale : NULL;
    P->Mn = ud->macro_mesh.no_nodes;
    P->Ne = ud->macro_mesh.no_elements;
    P->nv = ud->macro_mesh.no_verts;
    P->mn = ud->micro_mesh.no_nodes;
    P->mNe = ud->micro_mesh.no_elements;
    P->dirichlet = (unsigned char*)calloc((size_t)P->Mn, 1);
    if (ext && ext->n_templates > 0) {
        P->ntpl = ext->n_templates;
        P->tpl = ext->templates;
        P->cell_tpl = ext->cell_template;
    } else {
        P->ntpl = 1;
        P->tpl = &P->ud.micro_mesh;
        P->cell_tpl = NULL;
    }
    /* unknown offsets, scenario by scenario: [macro nodes of s | cells of
     * s, cell k following cell k-1]; one scenario is the reference layout */
    P->S = (ext && ext->scenarios > 1) ? ext->scenarios : 1;
    P->scen_nodes = P->Mn / P->S;
    P->scen_cells = P->Ne / P->S;
    P->learned = ext ? ext->cell_learned : NULL;
    P->kappa = ext ? ext->closure_coef : NULL;
    P->cell_off = (long*)malloc(sizeof(long) * (size_t)(P->Ne > 0 ? P->Ne : 1));
    P->node_off = (long*)malloc(sizeof(long) * (size_t)(P->Mn > 0 ? P->Mn : 1));
    P->scen_start = (long*)malloc(sizeof(long) * (size_t)(P->S + 1));
    long off = 0;
    for (int s = 0; s < P->S; ++s) {
        P->scen_start[s] = off;
        for (int i = s * P->scen_nodes; i < (s + 1) * P->scen_nodes; ++i) P->node_off[i] = off++;
        for (int k = s * P->scen_cells; k < (s + 1) * P->scen_cells; ++k) {
            P->cell_off[k] = off;
            off += (P->learned && P->learned[k]) ? 1 : P->tpl[P->cell_tpl ? P->cell_tpl[k] : 0].no_nodes;
        }
    }
    P->scen_start[P->S] = off;
    P->N = off;
    P->scen_pA = NULL;
    P->scen_kscale = NULL;
    if (ext && ext->scen_soilA) {
        P->scen_pA = (vgpar*)malloc(sizeof(vgpar) * (size_t)P->S);
        for (int s = 0; s < P->S; ++s) P->scen_pA[s] = make_vgpar(&ext->scen_soilA[s]);
    }
    if (ext && ext->scen_keff_scale) {
        P->scen_kscale = (double*)malloc(sizeof(double) * (size_t)P->S);
        for (int s = 0; s < P->S; ++s) P->scen_kscale[s] = ext->scen_keff_scale[s];
    }
    P->inv_Y = 1.0 / P->tpl[0].cell_area;
    P->cell_pB = NULL;
    if (ext && ext->cell_soilB) {
        P->cell_pB = (vgpar*)malloc(sizeof(vgpar) * (size_t)P->Ne);
        for (int k = 0; k < P->Ne; ++k) P->cell_pB[k] = make_vgpar(&ext->cell_soilB[k]);
    }
    /* face coefficients: (grad h) . n = D1 (h1 - h0) + D2 (h2 - h0) with
     * D_i = sfy_i ny + sfx_i nx (the gradient rows of the P1 interpolant
     * dotted with the length-weighted face normal), stored halved: the face
     * conductivity is the mean of two nodal values, (K_a + K_b)/2, and the
     * 1/2 rides on D (an exact scaling) */
    P->faceH = (double**)malloc(sizeof(double*) * (size_t)P->ntpl);
    P->max_mn = 0;
    P->max_mNe = 0;
    for (int t = 0; t < P->ntpl; ++t) {
        const micro_mesh_struct* mm = &P->tpl[t];
        const int mNe = mm->no_elements;
        if (mm->no_nodes > P->max_mn) P->max_mn = mm->no_nodes;
        if (mNe > P->max_mNe) P->max_mNe = mNe;
        P->faceH[t] = (double*)malloc(sizeof(double) * 6 * (size_t)mNe);
        for (int e = 0; e < mNe; ++e)
            for (int j = 0; j < 3; ++j) {
                double nx = mm->normals[(size_t)(2 * j) * mNe + e];
                double ny = mm->normals[(size_t)(2 * j + 1) * mNe + e];
                for (int i = 1; i <= 2; ++i)
                    P->faceH[t][(size_t)6 * e + 2 * j + i - 1] =
                        0.5 * fma(mm->shape_funcs[(size_t)(3 + i) * mNe + e], ny,
                                  mm->shape_funcs[(size_t)i * mNe + e] * nx);
            }
    }
    const macro_mesh_struct* M = &ud->macro_mesh;
    for (int k = 0; k < P->Ne; ++k)
        for (int j = 0; j < P->nv; ++j)
            if (M->boundary_condition_edges[j * P->Ne + k] == TSR_BC_DIRICHLET) {
                P->dirichlet[M->elements[j * P->Ne + k]] = 1;
                P->dirichlet[M->elements[((j + 1) % P->nv) * P->Ne + k]] = 1;
            }
    return P;
}

void oracle_destroy(oracle_problem* P)
{
    if (!P) return;
    free(P->dirichlet);
    for (int t = 0; t < P->ntpl; ++t) free(P->faceH[t]);
    free(P->faceH);
    free(P->cell_off);
    free(P->cell_pB);
    free(P->node_off);
    free(P->scen_start);
    free(P->scen_pA);
    free(P->scen_kscale);
    free(P->V); free(P->Hm); free(P->phi); free(P->g0); free(P->g1); free(P->w);
    free(P->unew); free(P->winv); free(P->x); free(P->D); free(P->Dt);
    free(P);
}

long oracle_num_unknowns(const oracle_problem* P) { return P->N; }

/* first unknown of scenario s (s = S gives N) */
long oracle_scenario_start(const oracle_problem* P, int s) { return P->scen_start[s]; }

int oracle_dirichlet_mask(const oracle_problem* P, unsigned char* out)
{
    memcpy(out, P->dirichlet, (size_t)P->Mn);
    return 0;
}

/* Macro interpolant coefficients of element k from node values H
 * (coefficient m of vertex i at shape_funcs[(m*nv+i)*Ne+k]; the same
 * contraction src/save_solution.cpp:273-283 performs). */
static void interp_coeffs(const oracle_problem* P, const double* H, int k, double al[4])
{
    const macro_mesh_struct* M = &P->ud.macro_mesh;
    int nv = P->nv, Ne = P->Ne;
    for (int m = 0; m < nv; ++m) {
        double a = M->shape_funcs[(size_t)(m * nv + 0) * Ne + k] * H[P->node_off[M->elements[k]]];
        for (int i = 1; i < nv; ++i)
            a = fma(M->shape_funcs[(size_t)(m * nv + i) * Ne + k],
                    H[P->node_off[M->elements[(size_t)i * Ne + k]]], a);
        al[m] = a;
    }
}

/* value of the macro interpolant at (x, y) (src/save_solution.cpp:304-314) */
static double interp_at(int nv, const double al[4], double x, double y)
{
    if (nv == 3) return fma(al[0], x, fma(al[1], y, al[2]));
    return fma(al[0], x, fma(al[1], y, fma(al[2], x * y, al[3])));
}

static void interp_grad(int nv, const double al[4], double x, double y, double* gx, double* gy)
{
    if (nv == 3) {
        *gx = al[0];
        *gy = al[1];
    } else {
        *gx = fma(al[2], y, al[0]);
        *gy = fma(al[2], x, al[1]);
    }
}

/* micro cell k: writes g of its micro nodes, returns the exchange inflow Q
 * into the inclusion.  x is the macro+micro state. */
static double micro_cell(const oracle_problem* P, const double* x, int k, double* g, double* scratch)
{
    const int t = P->cell_tpl ? P->cell_tpl[k] : 0;
    const micro_mesh_struct* m = &P->tpl[t];
    const macro_mesh_struct* M = &P->ud.macro_mesh;
    const int mn = m->no_nodes, mNe = m->no_elements, Ne = P->Ne;
    const long off = P->cell_off[k];
    const vgpar* pB = P->cell_pB ? &P->cell_pB[k] : &P->pB;
    const double s = P->cell_scale ? P->cell_scale[k] : 1.0;
    const double s2 = s * s;
    double* psi = scratch;
    double* Kn = scratch + mn;
    double* Cn = scratch + 2 * mn;
    double* Cd = scratch + 3 * mn;
    double* acc = scratch + 4 * mn;
    double* items = scratch + 5 * mn;
    int nitems = 0;
    double al[4];
    interp_coeffs(P, x, k, al);
    const double cx = M->centroid_elements[k], cy = M->centroid_elements[Ne + k];
    if (P->learned && P->learned[k]) {
        /* learned closure: one unknown, the interior mean water content th,
         * relaxing towards the water content theta_B(H_c) of the macro head
         * at the cell centre */
        const double th = x[off];
        const double Hc = interp_at(P->nv, al, cx, cy);
        double K, Cn, Cd, Se;
        vg_eval(Hc, pB, &K, &Cn, &Cd, &Se);
        const double d = fma(pB->dth, Se, pB->thr) - th;
        const double kQ = P->kappa ? P->kappa[2 * k] : 0.0;
        const double kT = P->kappa ? P->kappa[2 * k + 1] : 0.0;
        g[off] = kT * d;
        return kQ * d;
    }
    for (int l = 0; l < mn; ++l) {
        double hl;
        if (m->boundary_nodes[l] == 1) {
            /* micro boundary = macro interpolant (src/save_solution.cpp:285-315) */
            double px, py;
            if (P->ud.model_type == 1) {
                px = cx;
                py = cy;
            } else {
                px = fma(s, m->vectors[l], cx);
                py = fma(s, m->vectors[mn + l], cy);
            }
            hl = interp_at(P->nv, al, px, py);
        } else {
            hl = x[off + l];
        }
        double K, Se;
        vg_eval(hl, pB, &K, &Cn[l], &Cd[l], &Se);
        /* total head psi = h + y, with y the node's template height scaled
         * by s: for the P1 interpolant, grad(h + y) = grad h + e_y, so the
         * gravity term rides on the head differences */
        psi[l] = fma(s, m->vectors[mn + l], hl);
        Kn[l] = K;
        acc[l] = 0.0;
    }
    const int exch = (P->ud.model_type == 3);
    for (int e = 0; e < mNe; ++e) {
        int v[3];
        for (int j = 0; j < 3; ++j) v[j] = m->elements[(size_t)j * mNe + e];
        /* (grad h + e_y).n / 2 = (grad psi).n / 2 through the halved face
         * coefficients; a cell scaled by s about the template has gradient
         * grad/s and normals s n, so D is scale-free and the scale enters
         * through psi's height term only */
        double d1 = psi[v[1]] - psi[v[0]];
        double d2 = psi[v[2]] - psi[v[0]];
        const double* H = P->faceH[t] + (size_t)6 * e;
        for (int j = 0; j < 3; ++j) {
            int a = v[j], b = v[(j + 1) % 3];
            double dot = fma(H[2 * j + 1], d2, H[2 * j] * d1);
            double Kf;
            if (P->kface == 1)
                Kf = tsr_gt0(dot) ? Kn[b] : Kn[a];        /* upwind: 2 K (dot/2) */
            else
                Kf = Kn[a] + Kn[b];                       /* (K_a + K_b)/2 (2 dot/2) */
            double Pf = Kf * dot;           /* flow into SCV(a) from SCV(b) */
            acc[a] += Pf;
            acc[b] -= Pf;
        }
        if (exch) {
            for (int j = 0; j < 3; ++j) {
                if (m->boundary_edges[(size_t)j * mNe + e] != 1) continue;
                for (int sh = 0; sh < 2; ++sh) {
                    int vv = v[(j + sh) % 3];
                    double nbx = m->boundary_edge_normals[(size_t)(4 * j + 2 * sh) * mNe + e];
                    double nby = m->boundary_edge_normals[(size_t)(4 * j + 2 * sh + 1) * mNe + e];
                    double Db1 = fma(m->shape_funcs[(size_t)4 * mNe + e], nby,
                                     m->shape_funcs[(size_t)1 * mNe + e] * nbx);
                    double Db2 = fma(m->shape_funcs[(size_t)5 * mNe + e], nby,
                                     m->shape_funcs[(size_t)2 * mNe + e] * nbx);
                    items[nitems++] = Kn[vv] * fma(Db2, d2, Db1 * d1);
                }
            }
        }
    }
    for (int l = 0; l < mn; ++l) {
        if (m->boundary_nodes[l] == 1) {
            g[off + l] = 0.0;
        } else {
            double A = m->CV_area[l] * s2;
            double den = fma(P->Ss, Cd[l], Cn[l]) * A;
            g[off + l] = (acc[l] * Cd[l]) / den;
        }
    }
    double Q = 0.0;
    if (exch) {
        double p[32];
        for (int l = 0; l < 32; ++l) p[l] = 0.0;
        for (int i = 0; i < nitems; ++i) p[i & 31] += items[i];
        Q = butterfly32(p);
    }
    return Q;
}

static size_t scratch_doubles(const oracle_problem* P)
{
    return (size_t)5 * P->max_mn + (size_t)6 * P->max_mNe + 64;
}

/* g = G(x).  nthreads > 1: the micro cells run as an OpenMP loop (the
 * Gfunc_parallel form); the macro assembly is sequential in element order.
 * Returns 0, or 1 if G has a non-finite entry (the reference's Gfunc flag
 * convention: 0 = success). */
int oracle_g(oracle_problem* P, const double* x, double* g, int nthreads)
{
    const macro_mesh_struct* M = &P->ud.macro_mesh;
    const int Ne = P->Ne, Mn = P->Mn, nv = P->nv;
    double* Q = (double*)malloc(sizeof(double) * (size_t)Ne);
    size_t sd = scratch_doubles(P);
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
    {
        double* scratch = (double*)malloc(sizeof(double) * sd);
#pragma omp for schedule(static)
        for (int k = 0; k < Ne; ++k) Q[k] = micro_cell(P, x, k, g, scratch);
        free(scratch);
    }
#else
    (void)nthreads;
    {
        double* scratch = (double*)malloc(sizeof(double) * sd);
        for (int k = 0; k < Ne; ++k) Q[k] = micro_cell(P, x, k, g, scratch);
        free(scratch);
    }
#endif
    /* macro CVFE assembly, element by element: SCV faces, then boundary
     * sub-edges, then the exchange term, each scattered to its nodes */
    double* acc = (double*)calloc((size_t)Mn, sizeof(double));
    for (int k = 0; k < Ne; ++k) {
        int v[4];
        for (int j = 0; j < nv; ++j) v[j] = M->elements[(size_t)j * Ne + k];
        double al[4];
        interp_coeffs(P, x, k, al);
        for (int j = 0; j < nv; ++j) {
            double mx = M->midx[(size_t)j * Ne + k], my = M->midy[(size_t)j * Ne + k];
            double gx, gy;
            interp_grad(nv, al, mx, my, &gx, &gy);
            double Hf = interp_at(nv, al, mx, my);
            double K[4];
            keff_eval(Hf, &P->kp, K);
            if (P->scen_kscale)
                for (int q = 0; q < 4; ++q) K[q] *= P->scen_kscale[k / P->scen_cells];
            double gy1 = gy + 1.0;
            double qx = fma(K[0], gx, K[1] * gy1);
            double qy = fma(K[2], gx, K[3] * gy1);
            double nx = M->normals[(size_t)(2 * j) * Ne + k];
            double ny = M->normals[(size_t)(2 * j + 1) * Ne + k];
            double Pf = fma(qx, nx, qy * ny);
            acc[v[j]] += Pf;
            acc[v[(j + 1) % nv]] -= Pf;
        }
        for (int j = 0; j < nv; ++j) {
            int bc = M->boundary_condition_edges[(size_t)j * Ne + k];
            if (bc != TSR_BC_FLUX && bc != TSR_BC_DHDX0 && bc != TSR_BC_DHDY0) continue;
            for (int sh = 0; sh < 2; ++sh) {
                int vv = v[(j + sh) % nv];
                if (bc == TSR_BC_FLUX) {
                    acc[vv] += P->ud.boundary_flux * M->boundary_edge_lens[(size_t)(2 * j + sh) * Ne + k];
                } else {
                    double bx = M->boundary_edge_midpts[(size_t)(4 * j + 2 * sh) * Ne + k];
                    double by = M->boundary_edge_midpts[(size_t)(4 * j + 2 * sh + 1) * Ne + k];
                    double gx, gy;
                    interp_grad(nv, al, bx, by, &gx, &gy);
                    if (bc == TSR_BC_DHDX0) gx = 0.0;
                    if (bc == TSR_BC_DHDY0) gy = 0.0;
                    double Hb = interp_at(nv, al, bx, by);
                    double K[4];
                    keff_eval(Hb, &P->kp, K);
                    if (P->scen_kscale)
                        for (int q = 0; q < 4; ++q) K[q] *= P->scen_kscale[k / P->scen_cells];
                    double gy1 = gy + 1.0;
                    double qx = fma(K[0], gx, K[1] * gy1);
                    double qy = fma(K[2], gx, K[3] * gy1);
                    double nbx = M->boundary_edge_normals[(size_t)(4 * j + 2 * sh) * Ne + k];
                    double nby = M->boundary_edge_normals[(size_t)(4 * j + 2 * sh + 1) * Ne + k];
                    acc[vv] += fma(qx, nbx, qy * nby);
                }
            }
        }
        if (P->ud.model_type == 3) {
            /* inclusion uptake per unit area, distributed over the SCVs */
            double qk = Q[k] * P->inv_Y;
            for (int j = 0; j < nv; ++j) acc[v[j]] -= M->SCV_area[(size_t)j * Ne + k] * qk;
        }
    }
    for (int i = 0; i < Mn; ++i) {
        const long o = P->node_off[i];
        if (P->dirichlet[i]) {
            g[o] = 0.0;
            continue;
        }
        const vgpar* pA = P->scen_pA ? &P->scen_pA[i / P->scen_nodes] : &P->pA;
        double K, Cn, Cd, Se;
        vg_eval(x[o], pA, &K, &Cn, &Cd, &Se);
        double A = P->epsA * M->CV_area[i];
        double den = fma(P->Ss, Cd, Cn) * A;
        g[o] = (acc[i] * Cd) / den;
    }
    free(acc);
    free(Q);
    /* failure flag of the reference's Gfunc convention: non-zero when any
     * entry of G is not finite */
    for (long i = 0; i < P->N; ++i)
        if (!isfinite(g[i])) return 1;
    return 0;
}

/* w = (G(u + eps v) - g0) * (1/eps) */
int oracle_jv(oracle_problem* P, const double* u, const double* g0, const double* v,
              double eps, double* w, int nthreads)
{
    long N = P->N;
    double* x = (double*)malloc(sizeof(double) * (size_t)N);
    double* gx = (double*)malloc(sizeof(double) * (size_t)N);
    const int nt = nthreads > 1 ? nthreads : 1;
#pragma omp parallel for num_threads(nt) schedule(static) if (nt > 1)
    for (long i = 0; i < N; ++i) x[i] = fma(eps, v[i], u[i]);
    int rc = oracle_g(P, x, gx, nthreads);
    double inv = 1.0 / eps;
#pragma omp parallel for num_threads(nt) schedule(static) if (nt > 1)
    for (long i = 0; i < N; ++i) w[i] = (gx[i] - g0[i]) * inv;
    free(x);
    free(gx);
    return rc;
}

/* Water terms laid out scenario by scenario, [macro nodes of s | cells of
 * s] (one scenario: Mn node terms then Ne cell terms); per-scenario sums
 * go to per[s] when per is not NULL. */
static int water_terms(oracle_problem* P, const double* u, double* water, double* per)
{
    const macro_mesh_struct* M = &P->ud.macro_mesh;
    const int Mn = P->Mn, Ne = P->Ne, nv = P->nv;
    double* terms = (double*)malloc(sizeof(double) * (size_t)(Mn + Ne));
    for (int i = 0; i < Mn; ++i) {
        const vgpar* pA = P->scen_pA ? &P->scen_pA[i / P->scen_nodes] : &P->pA;
        double K, Cn, Cd, Se;
        vg_eval(u[P->node_off[i]], pA, &K, &Cn, &Cd, &Se);
        const int sc = i / P->scen_nodes;
        terms[(size_t)sc * (P->scen_nodes + P->scen_cells) + (i - sc * P->scen_nodes)] =
            (P->epsA * M->CV_area[i]) * fma(pA->dth, Se, pA->thr);
    }
    for (int k = 0; k < Ne; ++k) {
        const double s = P->cell_scale ? P->cell_scale[k] : 1.0;
        const micro_mesh_struct* m = &P->tpl[P->cell_tpl ? P->cell_tpl[k] : 0];
        const int mn = m->no_nodes;
        const vgpar* pB = P->cell_pB ? &P->cell_pB[k] : &P->pB;
        double al[4];
        interp_coeffs(P, u, k, al);
        double cx = M->centroid_elements[k], cy = M->centroid_elements[Ne + k];
        double p[32];
        for (int l = 0; l < 32; ++l) p[l] = 0.0;
        for (int l = 0; l < mn; ++l) {
            double hl;
            if (m->boundary_nodes[l] == 1) {
                double px = cx, py = cy;
                if (P->ud.model_type != 1) {
                    px = fma(s, m->vectors[l], cx);
                    py = fma(s, m->vectors[mn + l], cy);
                }
                hl = interp_at(nv, al, px, py);
            } else if (P->learned && P->learned[k]) {
                p[l & 31] += u[P->cell_off[k]] * m->CV_area[l];
                continue;
            } else {
                hl = u[P->cell_off[k] + l];
            }
            double K, Cn, Cd, Se;
            vg_eval(hl, pB, &K, &Cn, &Cd, &Se);
            p[l & 31] += fma(pB->dth, Se, pB->thr) * m->CV_area[l];
        }
        double area = M->SCV_area[k];
        for (int j = 1; j < nv; ++j) area += M->SCV_area[(size_t)j * Ne + k];
        const int sc = k / P->scen_cells;
        terms[(size_t)sc * (P->scen_nodes + P->scen_cells) + P->scen_nodes + (k - sc * P->scen_cells)] =
            (area * P->inv_Y) * ((s * s) * butterfly32(p));
    }
    *water = oracle_vsum(terms, (long)Mn + Ne);
    if (per)
        for (int sc = 0; sc < P->S; ++sc)
            per[sc] = oracle_vsum(terms + (size_t)sc * (P->scen_nodes + P->scen_cells),
                                  (long)P->scen_nodes + P->scen_cells);
    free(terms);
    return 0;
}

/* total water content */
int oracle_water(oracle_problem* P, const double* u, double* water)
{
    return water_terms(P, u, water, NULL);
}

/* water content of each scenario (S doubles) */
int oracle_water_scenarios(oracle_problem* P, const double* u, double* per)
{
    double total;
    return water_terms(P, u, &total, per);
}

/* ------------------------------------------------------------------ */
/* phi_1 by the (6,6) Pade approximant with scaling and squaring
 * (src/phipade.cpp:15-216; Hochbruck, Lubich & Selhofer 1998, p. 1567).
 * Deviation recorded: for m = 1 with exp(A) == 1 the reference returns 0
 * (and NaN for A == 0, src/phipade.cpp:32-40); phi_1 tends to 1 there and
 * this restatement returns 1.                                              */

static void o_matmul(int m, const double* A, const double* B, double* C)
{
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) {
            double c = 0.0;
            for (int k = 0; k < m; ++k) c = fma(A[k * m + i], B[j * m + k], c);
            C[j * m + i] = c;
        }
}

int oracle_phipade(double* phiH, const double* H, double alpha, int m, int ldH, int ldP)
{
    if (m < 1) return 5;
    if (m == 1) {
        double A = alpha * H[0];
        double eA = exp(A);
        if (eA == 1.0) phiH[0] = 1.0;
        else if (eA == 0.0) phiH[0] = -1.0 / A;
        else phiH[0] = ((eA - 1.0) * A / log(eA)) / A;
        return 0;
    }
    static const double a[6] = {1.0 / 26.0, 5.0 / 156.0, 1.0 / 858.0,
                                1.0 / 5720.0, 1.0 / 205920.0, 1.0 / 8648640.0};
    static const double b[6] = {-6.0 / 13.0, 5.0 / 52.0, -5.0 / 429.0,
                                1.0 / 1144.0, -1.0 / 25740.0, 1.0 / 1235520.0};
    int mm = m * m;
    double* buf = (double*)malloc(sizeof(double) * 6 * (size_t)mm);
    double *A = buf, *Pw = buf + mm, *D = buf + 2 * mm, *F = buf + 3 * mm, *E = buf + 4 * mm,
           *Tm = buf + 5 * mm;
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) A[j * m + i] = alpha * H[j * ldH + i];
    double nrm = 0.0;
    for (int i = 0; i < m; ++i) {
        double s = 0.0;
        for (int j = 0; j < m; ++j) s += fabs(A[j * m + i]);
        if (s > nrm || s != s) nrm = s;
    }
    int scale = 0;
    if (nrm > 0.0) {
        double sc = ceil(1.0 + log(nrm) / log(2.0));
        scale = sc > 0.0 ? (int)sc : 0;
    }
    if (scale > 0) {
        double f = 1.0 / pow(2.0, (double)scale);
        for (int i = 0; i < mm; ++i) A[i] *= f;
    }
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) {
            double d = (i == j) ? 1.0 : 0.0;
            F[j * m + i] = d;
            D[j * m + i] = d;
            E[j * m + i] = d;
        }
    memcpy(Pw, A, sizeof(double) * (size_t)mm);
    for (int i = 0; i < mm; ++i) {
        F[i] = fma(a[0], Pw[i], F[i]);
        D[i] = fma(b[0], Pw[i], D[i]);
    }
    for (int p = 1; p < 6; ++p) {
        o_matmul(m, Pw, A, Tm);
        memcpy(Pw, Tm, sizeof(double) * (size_t)mm);
        for (int i = 0; i < mm; ++i) {
            F[i] = fma(a[p], Pw[i], F[i]);
            D[i] = fma(b[p], Pw[i], D[i]);
        }
    }
    for (int k = 0; k < m; ++k) {
        int p = k;
        double best = fabs(D[k * m + k]);
        for (int i = k + 1; i < m; ++i)
            if (fabs(D[k * m + i]) > best) {
                best = fabs(D[k * m + i]);
                p = i;
            }
        if (!(best > 0.0)) {
            free(buf);
            return 7;
        }
        if (p != k) {
            for (int j = 0; j < m; ++j) {
                double t = D[j * m + k]; D[j * m + k] = D[j * m + p]; D[j * m + p] = t;
                t = F[j * m + k]; F[j * m + k] = F[j * m + p]; F[j * m + p] = t;
            }
        }
        double inv = 1.0 / D[k * m + k];
        for (int i = k + 1; i < m; ++i) {
            double l = D[k * m + i] * inv;
            D[k * m + i] = l;
            for (int j = k + 1; j < m; ++j) D[j * m + i] = fma(-l, D[j * m + k], D[j * m + i]);
            for (int j = 0; j < m; ++j) F[j * m + i] = fma(-l, F[j * m + k], F[j * m + i]);
        }
    }
    for (int j = 0; j < m; ++j)
        for (int i = m - 1; i >= 0; --i) {
            double s = F[j * m + i];
            for (int k = i + 1; k < m; ++k) s = fma(-D[k * m + i], F[j * m + k], s);
            F[j * m + i] = s / D[i * m + i];
        }
    if (scale > 0) {
        o_matmul(m, A, F, Tm);
        for (int i = 0; i < mm; ++i) E[i] += Tm[i];
        for (int it = 0; it < scale; ++it) {
            if (it > 0) {
                o_matmul(m, E, E, Tm);
                memcpy(E, Tm, sizeof(double) * (size_t)mm);
            }
            o_matmul(m, E, F, Tm);
            for (int i = 0; i < mm; ++i) F[i] = 0.5 * (Tm[i] + F[i]);
        }
    }
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) phiH[j * ldP + i] = F[j * m + i];
    free(buf);
    return 0;
}

/* ------------------------------------------------------------------ */
/* EXPREM: one accepted step of the Jacobian-free exponential
 * Rosenbrock-Euler method
 *     u+ = u + dt phi_1(dt J) G(u),  phi_1(dt J) G(u) ~ beta V_m phi_1(dt H_m) e1
 * with J v ~ (G(u + eps v) - G(u)) / eps, eps = sqrt((1 + ||u||_2) 2^-52),
 * the Krylov basis V built by Arnoldi with modified Gram-Schmidt.
 * Krylov dimension: grown from MinKrylov until the a-posteriori estimate
 *     errK = |dt beta h_{m+1,m} [phi_1(dt H_m)]_{m,1}| ||v_{m+1}||_w
 * is <= 0.1 (a tenth of the step tolerance); at MaxKrylov the step is
 * halved (at most by MinStepDecFac) on the same basis until it passes.
 * Step error: with D = G(u+) - G(u) - J(u+ - u), where J(u+ - u) is read off
 * the Arnoldi relation J V_m = V_{m+1} Hbar_m, the local error of the method
 * is 2 dt phi_3(dt J) D ~ (dt/3) D; it is measured in the weighted RMS norm
 *     ||e||_w = sqrt( (1/N) sum_i (e_i / (AbsTol + RelTol |u_i|))^2 )
 * (weighted_norm, include/exprem.h:27) and the step is accepted when <= 1.
 * Step control: dt <- dt * clamp(SafetyFac err^(-1/3), MinStepDecFac,
 * MaxStepIncFac), within [MinStep, MaxStep], clipped to reach tend.
 * A rejected step retries on the same Krylov basis (it does not depend on
 * dt).  Every tspan time crossed is filled by dense output
 *     u(t + tau) = u + tau beta V_m phi_1(tau H_m) e1.
 * stats.CurrentStep holds the step proposed for the next call.            */

static int alloc_workspace(oracle_problem* P, int maxk)
{
    if (P->V && P->maxk >= maxk) return 0;
    long N = P->N;
    free(P->V); free(P->Hm); free(P->phi); free(P->g0); free(P->g1); free(P->w);
    free(P->unew); free(P->winv); free(P->x); free(P->D); free(P->Dt);
    P->maxk = maxk;
    P->V = (double*)malloc(sizeof(double) * (size_t)N * (size_t)(maxk + 1));
    P->Hm = (double*)calloc((size_t)(maxk + 1) * (size_t)maxk, sizeof(double));
    P->phi = (double*)calloc((size_t)maxk * (size_t)maxk, sizeof(double));
    P->g0 = (double*)malloc(sizeof(double) * (size_t)N);
    P->g1 = (double*)malloc(sizeof(double) * (size_t)N);
    P->w = (double*)malloc(sizeof(double) * (size_t)N);
    P->unew = (double*)malloc(sizeof(double) * (size_t)N);
    P->winv = (double*)malloc(sizeof(double) * (size_t)N);
    P->x = (double*)malloc(sizeof(double) * (size_t)N);
    P->D = (double*)malloc(sizeof(double) * (size_t)N);
    P->Dt = (double*)malloc(sizeof(double) * (size_t)N);
    P->cache_valid = 0;
    return P->V ? 0 : 6;
}

/* u_out = u + sum_i c_i V_i, i ascending */
static void combine(const oracle_problem* P, const double* u, const double* c, int m, double* out)
{
    long N = P->N;
#pragma omp parallel for num_threads(o_threads) schedule(static) if (o_threads > 1)
    for (long l = 0; l < N; ++l) {
        double a = u[l];
        for (int i = 0; i < m; ++i) a = fma(c[i], P->V[(size_t)i * N + l], a);
        out[l] = a;
    }
}

/* Classical Gram-Schmidt twice (CGS2) of w against v_0..v_j: the
 * projections of w on every basis vector at once, w -= V c, the same again
 * with the projections d of the result, H(i, j) = c_i + d_i.  Every dot is
 * a fixed-order reduction (oracle_dot) and every update applies the basis
 * vectors in ascending order, one fused multiply-add each.  Two passes of
 * classical Gram-Schmidt keep the basis orthogonal to working accuracy
 * (Giraud, Langou, Rozloznik, Comput. Math. Appl. 50 (2005) 1069-1075,
 * "twice is enough"), with two global reductions of j+1 values instead of
 * the j+1 sequential ones of modified Gram-Schmidt. */
static void gs_cgs2(oracle_problem* P, int j, double* Hcol)
{
    const long N = P->N;
    const double* V = P->V;
    double* w = P->w;
    double c[512], d[512];
    for (int pass = 0; pass < 2; ++pass) {
        double* h = pass == 0 ? c : d;
        for (int i = 0; i <= j; ++i) h[i] = oracle_dot(w, V + (size_t)i * N, N);
#pragma omp parallel for num_threads(o_threads) schedule(static) if (o_threads > 1)
        for (long l = 0; l < N; ++l) {
            double y = w[l];
            for (int i = 0; i <= j; ++i) y = fma(-h[i], V[(size_t)i * N + l], y);
            w[l] = y;
        }
    }
    for (int i = 0; i <= j; ++i) Hcol[i] = c[i] + d[i];
}

int oracle_set_gram_schmidt(oracle_problem* P, int variant)
{
    if (!P || variant < 0 || variant > 1) return 1;
    P->gs_variant = variant;
    return 0;
}

#define KRYLOV_TOL 0.1

int oracle_exprem_step(oracle_problem* P, double* t_io, double tend, const double* tspan,
                       double* tspan_solns, double* u, const exprem_options_struct* opt,
                       exprem_stats_struct* st, int nthreads)
{
    const long N = P->N;
    const int maxk = opt->MaxKrylov < (int)N ? opt->MaxKrylov : (int)N;
    if (alloc_workspace(P, maxk)) return 6;
    o_threads = nthreads > 1 ? nthreads : 1;
    double t = *t_io;
    if (t == 0.0) {
        st->NumSteps = 0;
        st->FuncEvals = 0;
        st->CurrentStep = opt->InitStep;
        st->CurrentKryDim = 0;
        st->CurrentTime = 0.0;
        P->cache_valid = 0;
    }
    st->CurrentSoln = u;
    if (st->NumSteps >= opt->MaxNumSteps) return 9;
    double dt = st->CurrentStep;
    if (dt > opt->MaxStep) dt = opt->MaxStep;
    int last = 0;
    if (t + dt >= tend) {
        dt = tend - t;
        last = 1;
    }
    /* g0 = G(u), reused from the previous accepted step when the caller
     * passes back the same state */
    if (!(P->cache_valid && P->cache_u == u && P->cache_t == t)) {
        int flag = oracle_g(P, u, P->g0, nthreads);
        st->FuncEvals++;
        if (flag != 0) return 10;          /* G fails at the accepted state */
    }
    double* V = P->V;
    double* Hm = P->Hm;
    const int ldH = maxk + 1;
    memset(Hm, 0, sizeof(double) * (size_t)ldH * (size_t)maxk);
    /* weights of the error norm from the current state */
#pragma omp parallel for num_threads(o_threads) schedule(static) if (o_threads > 1)
    for (long l = 0; l < N; ++l) P->winv[l] = 1.0 / fma(opt->RelTol, fabs(u[l]), opt->AbsTol);
    const double beta = sqrt(oracle_dot(P->g0, P->g0, N));
    const double nu = sqrt(oracle_dot(u, u, N));
    const double eps = sqrt((1.0 + nu) * DBL_EPSILON);
    int m = 0, happy = 0;
    double errK = 0.0, vnw = 0.0;
    if (beta == 0.0) {
        /* stationary state: the step leaves u unchanged */
        m = 0;
    } else {
        double ib = 1.0 / beta;
#pragma omp parallel for num_threads(o_threads) schedule(static) if (o_threads > 1)
        for (long l = 0; l < N; ++l) V[l] = P->g0[l] * ib;
        for (int j = 0; j < maxk; ++j) {
            double* vj = V + (size_t)j * N;
            oracle_jv(P, u, P->g0, vj, eps, P->w, nthreads);
            st->FuncEvals++;
            double hs = 0.0;
            if (P->gs_variant == 1) {
                gs_cgs2(P, j, Hm + (size_t)j * ldH);
                for (int i = 0; i <= j; ++i) hs = fma(Hm[(size_t)j * ldH + i], Hm[(size_t)j * ldH + i], hs);
            } else {
                for (int i = 0; i <= j; ++i) {
                    double* vi = V + (size_t)i * N;
                    double hij = oracle_dot(P->w, vi, N);
                    Hm[(size_t)j * ldH + i] = hij;
                    hs = fma(hij, hij, hs);
#pragma omp parallel for num_threads(o_threads) schedule(static) if (o_threads > 1)
                    for (long l = 0; l < N; ++l) P->w[l] = fma(-hij, vi[l], P->w[l]);
                }
            }
            double hn = sqrt(oracle_dot(P->w, P->w, N));
            Hm[(size_t)j * ldH + j + 1] = hn;
            m = j + 1;
            if (!(hn > 1e-12 * sqrt(fma(hn, hn, hs)))) {
                happy = 1;
                break;
            }
            double ih = 1.0 / hn;
            double* vn = V + (size_t)(j + 1) * N;
#pragma omp parallel for num_threads(o_threads) schedule(static) if (o_threads > 1)
            for (long l = 0; l < N; ++l) vn[l] = P->w[l] * ih;
            if (m < opt->MinKrylov && m < maxk) continue;
            vnw = sqrt(oracle_wsq(vn, P->winv, N) / (double)N);
            if (oracle_phipade(P->phi, Hm, dt, m, ldH, maxk)) return 7;
            errK = fabs(((dt * beta) * hn) * P->phi[m - 1]) * vnw;
            if (errK <= KRYLOV_TOL) break;
        }
        if (!happy && errK > KRYLOV_TOL) {
            /* Krylov space too small for dt: shrink dt on the same basis */
            while (errK > KRYLOV_TOL) {
                double f = 0.5 > opt->MinStepDecFac ? 0.5 : opt->MinStepDecFac;
                dt = dt * f;
                last = 0;
                if (dt < opt->MinStep) return 8;
                if (oracle_phipade(P->phi, Hm, dt, m, ldH, maxk)) return 7;
                errK = fabs(((dt * beta) * Hm[(size_t)(m - 1) * ldH + m]) * P->phi[m - 1]) * vnw;
            }
        }
    }
    /* step attempts on the fixed basis */
    for (;;) {
        double c[512], z[513];
        double* unew = P->unew;
        if (m > 0) {
            if (oracle_phipade(P->phi, Hm, dt, m, ldH, maxk)) return 7;
            double dtb = dt * beta;
            for (int i = 0; i < m; ++i) c[i] = dtb * P->phi[i];
            combine(P, u, c, m, unew);
        } else {
            memcpy(unew, u, sizeof(double) * (size_t)N);
        }
        int flag = oracle_g(P, unew, P->g1, nthreads);
        st->FuncEvals++;
        double err;
        if (flag != 0) {
            err = INFINITY;
        } else if (m == 0) {
            err = 0.0;
        } else {
            /* z = Hbar_m c; D = g1 - g0 - sum_{i<=m} z_i V_i */
            int mz = happy ? m : m + 1;
            for (int i = 0; i < mz; ++i) {
                double a = 0.0;
                for (int k = 0; k < m; ++k) a = fma(Hm[(size_t)k * ldH + i], c[k], a);
                z[i] = a;
            }
            double dt3 = dt / 3.0;
#pragma omp parallel for num_threads(o_threads) schedule(static) if (o_threads > 1)
            for (long l = 0; l < N; ++l) {
                double d = P->g1[l] - P->g0[l];
                for (int i = 0; i < mz; ++i) d = fma(-z[i], V[(size_t)i * N + l], d);
                P->D[l] = d * dt3;
            }
            err = sqrt(oracle_wsq(P->D, P->winv, N) / (double)N);
        }
        if (err <= 1.0) {
            /* dense output at every tspan time in (t, t+dt] */
            int ns = (int)tspan[0];
            double tn = last ? tend : t + dt;
            for (int k = 1; k <= ns; ++k) {
                if (tspan[k] > t && tspan[k] <= tn) {
                    double* row = tspan_solns + (size_t)k * N;
                    if (m == 0) {
                        memcpy(row, u, sizeof(double) * (size_t)N);
                    } else {
                        double tau = tspan[k] - t;
                        if (oracle_phipade(P->phi, Hm, tau, m, ldH, maxk)) return 7;
                        double tb = tau * beta;
                        for (int i = 0; i < m; ++i) c[i] = tb * P->phi[i];
                        combine(P, u, c, m, row);
                    }
                }
            }
            memcpy(u, unew, sizeof(double) * (size_t)N);
            memcpy(P->g0, P->g1, sizeof(double) * (size_t)N);
            t = tn;
            double fac = (err > 0.0) ? opt->SafetyFac * pow(err, -1.0 / 3.0) : opt->MaxStepIncFac;
            if (fac > opt->MaxStepIncFac) fac = opt->MaxStepIncFac;
            if (fac < opt->MinStepDecFac) fac = opt->MinStepDecFac;
            double dn = dt * fac;
            if (dn > opt->MaxStep) dn = opt->MaxStep;
            if (dn < opt->MinStep) dn = opt->MinStep;
            st->CurrentStep = dn;
            st->CurrentTime = t;
            st->CurrentKryDim = m;
            st->NumSteps++;
            *t_io = t;
            P->cache_u = u;
            P->cache_t = t;
            P->cache_valid = 1;
            return 0;
        }
        /* reject: shrink and retry on the same basis */
        double fac = (err == err && err < INFINITY) ? opt->SafetyFac * pow(err, -1.0 / 3.0)
                                                     : opt->MinStepDecFac;
        if (fac < opt->MinStepDecFac) fac = opt->MinStepDecFac;
        if (fac > 1.0) fac = opt->MinStepDecFac;
        dt = dt * fac;
        last = 0;
        if (dt < opt->MinStep) return 8;
    }
}

/* ------------------------------------------------------------------ */
/* elementary functions, exported for their tests */
/* Per-cell summary of state u with g = G(u) (5 doubles per cell): macro
 * head at the cell centre H_c, interior mean water content theta (weights
 * CV areas), its rate sum C(h) g A / sum A, the exchange inflow Q and the
 * head h(theta) of the inverse retention curve.  Lane-ordered sums (item l
 * to lane l mod 32, then the xor butterfly).  Learned cells report their
 * unknown and closure values. */
int oracle_cell_summary(oracle_problem* P, const double* u, const double* g, double* out)
{
    const macro_mesh_struct* M = &P->ud.macro_mesh;
    const int Ne = P->Ne;
    double* gs = (double*)malloc(sizeof(double) * (size_t)P->N);
    double* scratch = (double*)malloc(sizeof(double) * scratch_doubles(P));
    for (int k = 0; k < Ne; ++k) {
        const micro_mesh_struct* m = &P->tpl[P->cell_tpl ? P->cell_tpl[k] : 0];
        const vgpar* pB = P->cell_pB ? &P->cell_pB[k] : &P->pB;
        double al[4];
        interp_coeffs(P, u, k, al);
        const double Hc = interp_at(P->nv, al, M->centroid_elements[k], M->centroid_elements[Ne + k]);
        const double Q = micro_cell(P, u, k, gs, scratch);
        double th, rate;
        if (P->learned && P->learned[k]) {
            th = u[P->cell_off[k]];
            rate = g[P->cell_off[k]];
        } else {
            double pw[32], pt[32], pr[32];
            for (int l = 0; l < 32; ++l) pw[l] = pt[l] = pr[l] = 0.0;
            for (int l = 0; l < m->no_nodes; ++l) {
                if (m->boundary_nodes[l] == 1) continue;
                const double h = u[P->cell_off[k] + l];
                double K, Cn, Cd, Se;
                vg_eval(h, pB, &K, &Cn, &Cd, &Se);
                const double A = m->CV_area[l];
                pw[l & 31] += A;
                pt[l & 31] += fma(pB->dth, Se, pB->thr) * A;
                pr[l & 31] += ((Cn / Cd) * g[P->cell_off[k] + l]) * A;
            }
            const double W = butterfly32(pw);
            th = butterfly32(pt) / W;
            rate = butterfly32(pr) / W;
        }
        double* o = out + (size_t)5 * k;
        o[0] = Hc;
        o[1] = th;
        o[2] = rate;
        o[3] = Q;
        o[4] = vg_head(th, pB);
    }
    free(gs);
    free(scratch);
    return 0;
}

double oracle_vg_head(const soil_struct* s, double theta)
{
    vgpar p = make_vgpar(s);
    return vg_head(theta, &p);
}

double oracle_math_log(double x) { return tsr_log(x, &T); }
double oracle_math_exp(double x) { return tsr_exp(x, &T); }
double oracle_math_expm1(double x) { return tsr_expm1(x, &T); }
double oracle_math_log1p(double x) { return tsr_log1p(x, &T); }
double oracle_math_log1p_unit(double x, double* s1) { return tsr_log1p_unit(x, s1, &T); }
/* the integer-pipe division over arrays (its test compares with IEEE a / b) */
void oracle_math_div_many(const double* a, const double* b, double* out, long n)
{
    for (long i = 0; i < n; ++i) out[i] = tsr_div(a[i], b[i], &T);
}

/* VG relations, exported for their tests: out = {K, C, theta} */
void oracle_vg(const soil_struct* s, double Ss, double h, double* out)
{
    vgpar p = make_vgpar(s);
    double K, Cn, Cd, Se;
    vg_eval(h, &p, &K, &Cn, &Cd, &Se);
    out[0] = K;
    out[1] = Cn / Cd + Ss;
    out[2] = fma(p.dth, Se, p.thr);
}

void oracle_keff(const Keff_struct* k, double H, double* K)
{
    keffpar kp;
    kp.n = k->no_hvalues;
    kp.first = k->logh_first;
    kp.inv_logr = 1.0 / k->logr;
    kp.Kv = k->Keff_values;
    keff_eval(H, &kp, K);
}
