// tsr_kernels.cu -- sm_103a kernels of the two-scale Richards hot path.
//
// Everything is FP64.  On GB300 the FP64 pipe (measured 0.50 Top/s for
// DFMA, DADD and DMUL alike) is ~70x slower than HBM per byte of the right-
// hand side, so the kernels are organised around FP64 instruction count:
//   * one persistent CTA per SM slot walks the micro cells; a cell's heads,
//     half-conductivities and face fluxes live in shared memory, and each
//     node gathers its face fluxes from a precomputed list (no atomics, a
//     fixed summation order, hence results independent of scheduling);
//   * elementary functions are the table-driven tsr_math.h routines (14
//     FP64 ops for log, 11 for exp, about half of the device libm's cost),
//     with their tables copied into shared memory once per CTA;
//   * transcendentals are evaluated once per node, never per face;
//   * the macro element terms ride on the CTA of the element's cell (cell k
//     belongs to macro element k), so one G costs two launches.
// All reductions use one fixed order (restated step by step in the oracle);
// the finite-difference Jv, the Gram-Schmidt coefficients
// and the step-error norm are therefore reproducible bit for bit.
//
// The code is compiled with -fmad=false: every fused multiply-add is an
// explicit fma(), matching the host evaluation operation for operation.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "tsr_device.h"
#include "tsr_internal.h"
#include "tsr_math.h"
#include "tsr_mlp.h"
#include "tsr_mlp_tc.cuh"

namespace tsr {

__device__ const tsr_math_tables d_tables = TSR_MATH_TABLES_INIT;

// host-side count of every kernel this library launches (a graph replay
// adds the kernels it contains; kernels recorded during capture are not
// launches)
static unsigned long long g_launches = 0;
static bool g_counting = true;
unsigned long long kernel_launches() { return g_launches; }
void add_launches(int n) { g_launches += (unsigned long long)n; }
void set_counting(bool on) { g_counting = on; }
static inline void count(int n = 1)
{
    if (g_counting) g_launches += (unsigned long long)n;
}

static constexpr int kTabDoubles = (int)(sizeof(tsr_math_tables) / sizeof(double));

__device__ __forceinline__ void load_tables(tsr_math_tables* s)
{
    const double2* src = reinterpret_cast<const double2*>(&d_tables);
    double2* dst = reinterpret_cast<double2*>(s);
    for (int i = threadIdx.x; i < (int)(sizeof(tsr_math_tables) / 16); i += blockDim.x) dst[i] = src[i];
}

__device__ __forceinline__ bool finite_d(double x)
{
    return (tsr_d2u(x) & TSR_ABS_MASK) < TSR_INF_BITS;
}

// ---- van Genuchten-Mualem (same operation sequence as the host oracle) ---
// sign tests and sign flips run on the bits (tsr_lt0 / tsr_ge0 / tsr_negate /
// tsr_negabs equal h < 0, nL >= 0, -h and -|nL| for every non-NaN value)
__device__ __forceinline__ void vg_full(double h, const VGPar& p, const tsr_math_tables* T,
                                        double& K, double& Cn, double& Cd)
{
    if (tsr_lt0(h)) {
        double ah = tsr_negate(h);
        double a = p.alpha * ah;
        double L = tsr_log(a, T);
        double nL = p.n * L;
        double e = tsr_exp(tsr_negabs(nL), T);      // min(t, 1/t)
        double s1;
        double lp = tsr_log1p_unit(e, &s1, T);
        const bool dry = tsr_ge0(nL);
        double l1 = dry ? nL + lp : lp;             // log(1+t)
        double y = dry ? -(p.m * lp) : p.m * (nL - lp);
        double X = tsr_exp(p.mh * l1, T);
        double Se = X * X;
        double B = -tsr_expm1(y, T);
        K = (p.Ks * X) * (B * B);
        Cn = dry ? p.coefC * Se : p.coefC * (e * Se);
        Cd = ah * s1;
    } else {
        K = p.Ks;
        Cn = 0.0;
        Cd = 1.0;
    }
}

__device__ __forceinline__ void vg_storage(double h, const VGPar& p, const tsr_math_tables* T,
                                           double& Cn, double& Cd)
{
    if (tsr_lt0(h)) {
        double ah = tsr_negate(h);
        double a = p.alpha * ah;
        double L = tsr_log(a, T);
        double nL = p.n * L;
        double e = tsr_exp(tsr_negabs(nL), T);
        double s1;
        double lp = tsr_log1p_unit(e, &s1, T);
        const bool dry = tsr_ge0(nL);
        double l1 = dry ? nL + lp : lp;
        double X = tsr_exp(p.mh * l1, T);
        double Se = X * X;
        Cn = dry ? p.coefC * Se : p.coefC * (e * Se);
        Cd = ah * s1;
    } else {
        Cn = 0.0;
        Cd = 1.0;
    }
}

__device__ __forceinline__ double vg_se(double h, const VGPar& p, const tsr_math_tables* T)
{
    if (!tsr_lt0(h)) return 1.0;
    double ah = tsr_negate(h);
    double a = p.alpha * ah;
    double L = tsr_log(a, T);
    double nL = p.n * L;
    double e = tsr_exp(tsr_negabs(nL), T);
    double s1;
    double lp = tsr_log1p_unit(e, &s1, T);
    double l1 = tsr_ge0(nL) ? nL + lp : lp;
    double X = tsr_exp(p.mh * l1, T);
    return X * X;
}

// head at water content theta (inverse retention curve; same operation
// sequence as the oracle's vg_head): 0 at or above saturation, Se >= 1e-12
__device__ __forceinline__ double vg_head(double theta, const VGPar& p, const tsr_math_tables* T)
{
    double Se = (theta - p.thr) / p.dth;
    if (!(Se < 1.0)) return 0.0;
    if (!(Se > 1e-12)) Se = 1e-12;
    double L = tsr_log(Se, T);
    double tt = tsr_expm1(-(L / p.m), T);
    double lt = tsr_log(tt, T);
    return -(tsr_exp(lt / p.n, T) / p.alpha);
}

// ---- effective conductivity table --------------------------------------
__device__ __forceinline__ void keff_dev(double H, const MacroDev& M, const tsr_math_tables* T,
                                         double K[4])
{
    const int n = M.nk;
    if (n < 2) {
        for (int c = 0; c < 4; ++c) K[c] = M.keff[c * n];
        return;
    }
    double x = tsr_log(fabs(H), T) * TSR_INV_LN10;
    double pos = (x - M.keff_first) * M.keff_inv_logr;
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
        double k0 = __ldg(M.keff + c * n + i), k1 = __ldg(M.keff + c * n + i + 1);
        K[c] = fma(w, k1 - k0, k0);
    }
}

__device__ __forceinline__ double interp_at(int nv, const double* al, double x, double y)
{
    if (nv == 3) return fma(al[0], x, fma(al[1], y, al[2]));
    return fma(al[0], x, fma(al[1], y, fma(al[2], x * y, al[3])));
}

__device__ __forceinline__ void interp_grad(int nv, const double* al, double x, double y,
                                            double& gx, double& gy)
{
    if (nv == 3) {
        gx = al[0];
        gy = al[1];
    } else {
        gx = fma(al[2], y, al[0]);
        gy = fma(al[2], x, al[1]);
    }
}

template <int MODE>
__device__ __forceinline__ double state_at(const double* __restrict__ u, const double* __restrict__ v,
                                           double eps, long long i)
{
    if (MODE == 0) return u[i];
    return fma(eps, v[i], u[i]);
}

// Macro element k's contributions (faces, boundary sub-edges, exchange),
// one per lane of warp 0.  Slot layout per element: [0,nv) faces,
// [nv,3nv) boundary halves (2j+s), [3nv,4nv) exchange.
__device__ __forceinline__ void macro_element_terms(const Problem& P, int k, const double* al, double Q,
                                    const tsr_math_tables* T, int lane)
{
    const MacroDev& M = P.M;
    const int nv = M.nv, Ne = M.Ne;
    // per-scenario factor on Keff (ensemble form)
    const double ks = M.scen_kscale ? M.scen_kscale[k / M.scen_cells] : 1.0;
    double* out = P.contrib + (long long)16 * k;
    if (lane < nv) {
        const int j = lane;
        double mx = M.midx[(long long)j * Ne + k], my = M.midy[(long long)j * Ne + k];
        double gx, gy;
        interp_grad(nv, al, mx, my, gx, gy);
        double Hf = interp_at(nv, al, mx, my);
        double K[4];
        keff_dev(Hf, M, T, K);
        if (M.scen_kscale)
            for (int q = 0; q < 4; ++q) K[q] *= ks;
        double gy1 = gy + 1.0;
        double qx = fma(K[0], gx, K[1] * gy1);
        double qy = fma(K[2], gx, K[3] * gy1);
        double nx = M.normals[(long long)(2 * j) * Ne + k];
        double ny = M.normals[(long long)(2 * j + 1) * Ne + k];
        out[j] = fma(qx, nx, qy * ny);
    } else if (lane < 3 * nv) {
        const int q = lane - nv, j = q >> 1, sh = q & 1;
        const int bc = M.bce[(long long)j * Ne + k];
        if (bc == 1) {
            out[nv + q] = M.bflux * M.blen[(long long)(2 * j + sh) * Ne + k];
        } else if (bc == 3 || bc == 4) {
            double bx = M.bmid[(long long)(4 * j + 2 * sh) * Ne + k];
            double by = M.bmid[(long long)(4 * j + 2 * sh + 1) * Ne + k];
            double gx, gy;
            interp_grad(nv, al, bx, by, gx, gy);
            if (bc == 3) gx = 0.0;
            if (bc == 4) gy = 0.0;
            double Hb = interp_at(nv, al, bx, by);
            double K[4];
            keff_dev(Hb, M, T, K);
            if (M.scen_kscale)
                for (int q = 0; q < 4; ++q) K[q] *= ks;
            double gy1 = gy + 1.0;
            double qx = fma(K[0], gx, K[1] * gy1);
            double qy = fma(K[2], gx, K[3] * gy1);
            double nbx = M.bnrm[(long long)(4 * j + 2 * sh) * Ne + k];
            double nby = M.bnrm[(long long)(4 * j + 2 * sh + 1) * Ne + k];
            out[nv + q] = fma(qx, nbx, qy * nby);
        }
    } else if (lane < 4 * nv) {
        if (M.model_type == 3) {
            const int j = lane - 3 * nv;
            out[3 * nv + j] = M.scv[(long long)j * Ne + k] * (Q * M.inv_Y);
        }
    }
}

// ---- the micro-cell kernel ----------------------------------------------
// A persistent CTA walks bundles: groups of cells that share one template
// (one cell per bundle for large templates, many for small ones, as packed
// by the host-side autotuner).  For a bundle of nc cells with mn nodes and
// mNe elements each, dynamic shared memory holds
//   tables | misc [slots x 16] | cell ids / offsets [slots] |
//   psi[nc mn] | K[nc mn] | Cd[nc mn] | den[nc mn] | F[nc 3 mNe] | items[nc nb]
// and the threads sweep the bundle's flattened node and element index
// spaces.  Every cell still follows the single-cell operation sequence (the
// same as the host oracle), so packing changes speed, never bits.
template <int MODE, bool STAB>
__global__ void __launch_bounds__(1024) k_cells(Problem P, const double* __restrict__ u,
                                                const double* __restrict__ v,
                                                const double* __restrict__ g0,
                                                const double* __restrict__ epsv,
                                                double* __restrict__ out)
{
    // The finite-difference step and its reciprocal come from device memory
    // (one pair per scenario) so that a captured graph replays with the
    // current values; cells of scenarios that are not active are skipped.
    // STAB: the math tables are copied into shared memory once per CTA;
    // otherwise they are read from global memory through L1 (14 KB less
    // shared memory per CTA, more CTAs per SM)
    extern __shared__ double sm[];
    const tsr_math_tables* T = STAB ? reinterpret_cast<const tsr_math_tables*>(sm) : &d_tables;
    double* misc = sm + (STAB ? kTabDoubles : 0);            // 16 per cell slot
    long long* coff = reinterpret_cast<long long*>(misc + 16 * P.misc_slots);
    int* ck = reinterpret_cast<int*>(coff + P.misc_slots);
    double* st = reinterpret_cast<double*>(ck + 2 * P.misc_slots);
    const int tid = threadIdx.x, bs = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarps = bs >> 5;
    const MacroDev& M = P.M;
    const MicroSet& S = P.m;
    const int nv = M.nv, Ne = M.Ne;
    const bool exch = (M.model_type == 3);
    if (STAB) {
        load_tables(reinterpret_cast<tsr_math_tables*>(sm));
        __syncthreads();
    }
    // The macro nodes' storage terms: their van Genuchten chains need only
    // the state, so they run here, beside the cells, and k_macro_nodes
    // keeps the gather and the division
    for (int i = blockIdx.x * bs + tid; i < M.Mn; i += gridDim.x * bs) {
        const int sc = M.nscen > 1 ? i / M.scen_nodes : 0;
        if ((P.active && !P.active[sc]) || M.dirichlet[i]) continue;
        const long long o = M.node_off ? M.node_off[i] : i;
        const double eps = MODE ? epsv[(long long)sc * P.eps_stride] : 0.0;
        const double H = state_at<MODE>(u, v, eps, o);
        double Cn, Cd;
        vg_storage(H, M.scen_pA ? M.scen_pA[sc] : P.pA, T, Cn, Cd);
        const double A = M.epsA * M.cv[i];
        P.node_st[2 * i] = Cd;
        P.node_st[2 * i + 1] = fma(M.Ss, Cd, Cn) * A;
    }
    int* cscen = ck + P.misc_slots;                          // scenario of each cell, -1 inactive
    for (int b = blockIdx.x; b < S.n_bundles; b += gridDim.x) {
        const int t = S.bundle_tpl[b], first = S.bundle_first[b], nc = S.bundle_count[b];
        if (P.active) {
            int any = 0;
            for (int c = tid; c < nc; c += bs) {
                const int k = S.bundle_cells[first + c];
                any |= P.active[M.nscen > 1 ? k / M.scen_cells : 0];
            }
            if (!__syncthreads_or(any)) continue;
        } else {
            __syncthreads();
        }
        const TplDesc D = S.tpl[t];
        const int mn = D.mn, mNe = D.mNe, nb = D.nb;
        double* h = st;                              // total heads psi = h + s y
        double* Kh = h + nc * mn;                    // nodal conductivities K(h)
        double* Cd = Kh + nc * mn;
        double* den = Cd + nc * mn;
        double* F = den + nc * mn;
        double* items = F + nc * 3 * mNe;
        const int* ev = S.ev + D.ev;
        const double* eg = S.eg + D.eg;
        const int* cptr = S.csr_ptr + D.csr_ptr;
        const int* cent = S.csr_ent + D.csr_ent;
        const int* bnode = S.bnode + D.node;
        const double* cvm = S.cv + D.node;
        const double* vec = S.vec + 2 * D.node;
        const int* bee = S.b_e + D.bitem;
        const int* bvv = S.b_v + D.bitem;
        const double* bnn = S.b_n + 2 * (long long)D.bitem;
        // per cell: id, first unknown, vertex heads and interpolant coefficients
        for (int c = warp; c < nc; c += nwarps) {
            const int k = S.bundle_cells[first + c];
            double* mc = misc + 16 * c;
            const int sc = M.nscen > 1 ? k / M.scen_cells : 0;
            const bool on = !P.active || P.active[sc];
            const double eps = MODE ? epsv[(long long)sc * P.eps_stride] : 0.0;
            if (lane == 0) {
                ck[c] = k;
                cscen[c] = on ? sc : -1;
                coff[c] = S.cell_off[k];
                mc[4] = P.cell_scale ? P.cell_scale[k] : 1.0;
                mc[7] = mc[4] * mc[4];
                mc[5] = M.cent[k];
                mc[6] = M.cent[Ne + k];
                mc[12] = eps;
                mc[13] = MODE ? epsv[(long long)sc * P.eps_stride + 1] : 0.0;
            }
            if (lane < nv) {
                long long vi = M.elements[(long long)lane * Ne + k];
                if (M.node_off) vi = M.node_off[vi];
                mc[8 + lane] = state_at<MODE>(u, v, eps, vi);
            }
            __syncwarp();
            if (lane < nv) {
                const int m = lane;
                double a = M.sf[(long long)(m * nv + 0) * Ne + k] * mc[8];
                for (int i = 1; i < nv; ++i)
                    a = fma(M.sf[(long long)(m * nv + i) * Ne + k], mc[8 + i], a);
                mc[m] = a;
            }
            __syncwarp();
            // heads of the inclusion-boundary nodes: the macro interpolant at
            // centroid + s vectors (model_type 1: at the centroid), one lane
            // per boundary node (dense; the node loop below only reads them)
            if (on && D.kind == 0) {
                const int* bl = S.bnl + D.bnl;
                const double s = mc[4];
                for (int q = lane; q < D.nbn; q += 32) {
                    const int l = bl[q];
                    double px = mc[5], py = mc[6];
                    if (M.model_type != 1) {
                        px = fma(s, vec[l], mc[5]);
                        py = fma(s, vec[mn + l], mc[6]);
                    }
                    h[c * mn + l] = interp_at(nv, mc, px, py);
                }
            }
        }
        __syncthreads();
        if (D.kind == 1) {
            // learned closure: one unknown per cell (interior mean water
            // content theta), inflow kQ (theta_B(H_c) - theta), rate
            // kT (theta_B(H_c) - theta)
            for (int c = warp; c < nc; c += nwarps) {
                if (cscen[c] < 0) continue;
                const int k = ck[c];
                const double* mc = misc + 16 * c;
                double Q = 0.0;
                if (lane == 0) {
                    const VGPar& pB = S.cell_par ? S.cell_par[k] : P.pB;
                    const double th = state_at<MODE>(u, v, mc[12], coff[c]);
                    const double Hc = interp_at(nv, mc, mc[5], mc[6]);
                    const double d = fma(pB.dth, vg_se(Hc, pB, T), pB.thr) - th;
                    const double g = S.kappa[2 * k + 1] * d;
                    Q = S.kappa[2 * k] * d;
                    if (!finite_d(g)) atomicOr(P.flag + cscen[c], 1);
                    const long long o = coff[c];
                    if (MODE == 0)
                        out[o] = g;
                    else
                        out[o] = (g - g0[o]) * mc[13];
                    if (MODE == 0 && P.qlog) P.qlog[k] = Q;
                }
                Q = __shfl_sync(0xffffffffu, Q, 0);
                macro_element_terms(P, k, mc, Q, T, lane);
            }
            continue;
        }
        // nodes: head, conductivity, storage
        for (int idx = tid; idx < nc * mn; idx += bs) {
            const int c = idx / mn, l = idx - c * mn;
            if (cscen[c] < 0) continue;
            const double* mc = misc + 16 * c;
            const double s = mc[4];
            const VGPar& pB = S.cell_par ? S.cell_par[ck[c]] : P.pB;
            const bool bnd = bnode[l] != 0;
            // boundary heads come from the per-cell pass above
            const double hl = bnd ? h[idx] : state_at<MODE>(u, v, mc[12], coff[c] + l);
            // total head: grad(h + y) = grad h + e_y for the P1 interpolant,
            // so the gravity term rides on the head differences (y is the
            // node's template height scaled by the cell's s)
            h[idx] = fma(s, vec[mn + l], hl);
            double K, Cn, Cdl;
            vg_full(hl, pB, T, K, Cn, Cdl);
            Kh[idx] = K;
            Cd[idx] = Cdl;
            den[idx] = fma(M.Ss, Cdl, Cn) * (cvm[l] * mc[7]);
        }
        __syncthreads();
        // elements: SCV face fluxes and inclusion-boundary exchange items
        for (int idx = tid; idx < nc * mNe; idx += bs) {
            const int c = idx / mNe, e = idx - c * mNe;
            if (cscen[c] < 0) continue;
            const double* hc = h + c * mn;
            const double* Khc = Kh + c * mn;
            const int v0 = ev[3 * e], v1 = ev[3 * e + 1], v2 = ev[3 * e + 2];
            const double* G = eg + 6 * (long long)e;   // per face: D1/2, D2/2
            const double h0 = hc[v0];
            const double d1 = hc[v1] - h0, d2 = hc[v2] - h0;
            const int vv[3] = {v0, v1, v2};
            double* Fc = F + (long long)c * 3 * mNe;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int a = vv[j], bb = vv[(j + 1) % 3];
                const double dot = fma(G[2 * j + 1], d2, G[2 * j] * d1);   // (grad psi . n)/2
                double Kf;
                if (P.kface == 1)
                    Kf = tsr_gt0(dot) ? Khc[bb] : Khc[a];
                else
                    Kf = Khc[a] + Khc[bb];
                Fc[3 * e + j] = Kf * dot;
            }
        }
        // inclusion-boundary exchange items, a dense loop of their own (as
        // part of the element loop they left most lanes of a warp idle):
        // K at the item's vertex times (grad psi . n_b) of its element
        if (exch) {
            for (int idx = tid; idx < nc * nb; idx += bs) {
                const int c = idx / nb, q = idx - c * nb;
                if (cscen[c] < 0) continue;
                const double* hc = h + c * mn;
                const int e = bee[q];
                const double h0 = hc[ev[3 * e]];
                const double d1 = hc[ev[3 * e + 1]] - h0, d2 = hc[ev[3 * e + 2]] - h0;
                const double* B = bnn + 2 * (long long)q;   // Db1, Db2
                items[idx] = Kh[c * mn + bvv[q]] * fma(B[1], d2, B[0] * d1);
            }
        }
        __syncthreads();
        // nodes: gather face fluxes in the fixed order, divide by storage
        for (int idx = tid; idx < nc * mn; idx += bs) {
            const int c = idx / mn, l = idx - c * mn;
            if (cscen[c] < 0) continue;
            double g;
            if (bnode[l]) {
                g = 0.0;
            } else {
                const double* Fc = F + (long long)c * 3 * mNe;
                double acc = 0.0;
                const int p1 = cptr[l + 1];
                for (int p = cptr[l]; p < p1; ++p) {
                    // acc - f is acc + (-f): the sign flip is a bit operation,
                    // so every entry costs one FP64 addition
                    const int ent = cent[p];
                    const double f = Fc[ent >> 1];
                    acc = acc + tsr_u2d(tsr_d2u(f) ^ ((uint64_t)(ent & 1) << 63));
                }
                g = tsr_div(acc * Cd[idx], den[idx], T);     // IEEE quotient, integer pipe
            }
            if (!finite_d(g)) atomicOr(P.flag + cscen[c], 1);
            const long long o = coff[c] + l;
            if (MODE == 0)
                out[o] = g;
            else
                out[o] = (g - g0[o]) * misc[16 * c + 13];
        }
        // exchange flux and the macro element terms: one warp per cell
        for (int c = warp; c < nc; c += nwarps) {
            if (cscen[c] < 0) continue;
            double Q = 0.0;
            if (exch) {
                const double* it = items + c * nb;
                double p = 0.0;
                for (int i = lane; i < nb; i += 32) p = p + it[i];
#pragma unroll
                for (int d = 16; d >= 1; d >>= 1) p = p + __shfl_xor_sync(0xffffffffu, p, d);
                Q = p;
            }
            if (MODE == 0 && P.qlog && lane == 0) P.qlog[ck[c]] = Q;
            macro_element_terms(P, ck[c], misc + 16 * c, Q, T, lane);
        }
    }
}

// ---- macro nodes ----------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(128) k_macro_nodes(Problem P, const double* __restrict__ u,
                                                     const double* __restrict__ v,
                                                     const double* __restrict__ g0,
                                                     const double* __restrict__ epsv,
                                                     double* __restrict__ out)
{
    // the storage terms (Cd, den) of every node come from the cell kernel
    const MacroDev& M = P.M;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.Mn) return;
    const int sc = M.nscen > 1 ? i / M.scen_nodes : 0;
    if (P.active && !P.active[sc]) return;
    const long long o = M.node_off ? M.node_off[i] : i;
    double g;
    if (M.dirichlet[i]) {
        g = 0.0;
    } else {
        double acc = 0.0;
        const int p1 = M.csr_ptr[i + 1];
        for (int p = M.csr_ptr[i]; p < p1; ++p) {
            const int ent = M.csr_ent[p];
            const double c = P.contrib[ent >> 1];
            acc = acc + tsr_u2d(tsr_d2u(c) ^ ((uint64_t)(ent & 1) << 63));
        }
        const double Cd = P.node_st[2 * i], den = P.node_st[2 * i + 1];
        g = (acc * Cd) / den;
    }
    if (!finite_d(g)) atomicOr(P.flag + sc, 1);
    if (MODE == 0)
        out[o] = g;
    else
        out[o] = (g - g0[o]) * epsv[(long long)sc * P.eps_stride + 1];
}

int configure_cell_kernels(const Problem& P, int* occ)
{
    cudaError_t e = cudaSuccess;
    for (auto f : {k_cells<0, true>, k_cells<1, true>, k_cells<0, false>, k_cells<1, false>})
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.micro_smem);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            occ, P.tables_smem ? k_cells<0, true> : k_cells<0, false>, P.micro_block, P.micro_smem);
    if (e != cudaSuccess) {
        set_error(std::string("configuring the cell kernel: ") + cudaGetErrorString(e));
        return 1;
    }
    if (*occ < 1) *occ = 1;
    return 0;
}

void launch_g(const Problem& P, int mode, const double* u, const double* v, const double* g0,
              const double* epsv, double* out, cudaStream_t s)
{
    const int nb = (P.M.Mn + 127) / 128;
    count(2);
    if (mode == 0) {
        if (P.tables_smem)
            k_cells<0, true><<<P.micro_grid, P.micro_block, P.micro_smem, s>>>(P, u, v, g0, epsv, out);
        else
            k_cells<0, false><<<P.micro_grid, P.micro_block, P.micro_smem, s>>>(P, u, v, g0, epsv, out);
        k_macro_nodes<0><<<nb, 128, 0, s>>>(P, u, v, g0, epsv, out);
    } else {
        if (P.tables_smem)
            k_cells<1, true><<<P.micro_grid, P.micro_block, P.micro_smem, s>>>(P, u, v, g0, epsv, out);
        else
            k_cells<1, false><<<P.micro_grid, P.micro_block, P.micro_smem, s>>>(P, u, v, g0, epsv, out);
        k_macro_nodes<1><<<nb, 128, 0, s>>>(P, u, v, g0, epsv, out);
    }
}

// ---- fixed-order reductions ------------------------------------------------
// Within a segment (a whole vector, or one scenario's part of it), block b
// covers items [8192 b, 8192 (b+1)) relative to the segment's start; thread t
// sums items 8192 b + 256 s + t (s ascending); warps combine by xor
// butterfly, the 8 warp sums as ((w0+w1)+(w2+w3))+((w4+w5)+(w6+w7)).  The
// last block of the segment to finish reduces its block sums the same way
// (thread t: P[t], P[t+256], ...).  A segment is therefore reduced exactly
// as it would be on its own.
static constexpr int kRedThreads = 256;
static constexpr int kRedChunk = 8192;

int reduction_blocks(long long n)
{
    long long b = (n + kRedChunk - 1) / kRedChunk;
    return (int)(b > 0 ? b : 1);
}

SegInfo single_segment(long long n, RedWork w)
{
    SegInfo g{};
    g.nseg = 1;
    g.nblocks = reduction_blocks(n);
    g.n1 = n;
    g.counters = w.counter;
    return g;
}

struct SegBlock {
    int s;          // segment
    long long lo;   // first item of the segment
    long long hi;   // one past its last item
    int lb;         // block index within the segment
    int b0;         // first block of the segment
    int nb;         // blocks of the segment
};

__device__ __forceinline__ SegBlock seg_block(const SegInfo& g)
{
    SegBlock r;
    if (g.start) {
        r.s = g.blkseg[blockIdx.x];
        r.lo = g.start[r.s];
        r.hi = g.start[r.s + 1];
        r.b0 = g.block0[r.s];
        r.nb = g.block0[r.s + 1] - r.b0;
        r.lb = (int)blockIdx.x - r.b0;
    } else {
        r.s = 0;
        r.lo = 0;
        r.hi = g.n1;
        r.b0 = 0;
        r.nb = (int)gridDim.x;
        r.lb = (int)blockIdx.x;
    }
    return r;
}

__device__ __forceinline__ double block_sum_256(double a, double* ws)
{
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) a = a + __shfl_xor_sync(0xffffffffu, a, d);
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) ws[warp] = a;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) r = ((ws[0] + ws[1]) + (ws[2] + ws[3])) + ((ws[4] + ws[5]) + (ws[6] + ws[7]));
    __syncthreads();
    return r;
}

// called by all threads with the block's partial sum (valid on thread 0)
__device__ __forceinline__ void finish_reduction(double r, const SegBlock& B, double* partials,
                                                 unsigned int* counter, double* res)
{
    __shared__ double ws[8];
    __shared__ int last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = r;
        __threadfence();
        unsigned int prev = atomicAdd(counter, 1u);
        last = (prev == (unsigned int)(B.nb - 1));
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double a = 0.0;
    for (int i = threadIdx.x; i < B.nb; i += kRedThreads) a = a + __ldcg(partials + B.b0 + i);
    double tot = block_sum_256(a, ws);
    if (threadIdx.x == 0) {
        *res = tot;
        *counter = 0u;
    }
}

template <class Term>
__global__ void __launch_bounds__(kRedThreads) k_reduce(Term term, SegInfo g, double* partials,
                                                        double* res, int rstride)
{
    __shared__ double ws[8];
    const SegBlock B = seg_block(g);
    if (g.active && !g.active[B.s]) return;
    const long long base = B.lo + (long long)B.lb * kRedChunk + threadIdx.x;
    double a = 0.0;
#pragma unroll 4
    for (int q = 0; q < kRedChunk / kRedThreads; ++q) {
        const long long i = base + (long long)q * kRedThreads;
        if (i < B.hi) a = term(B.s, i, a);
    }
    double r = block_sum_256(a, ws);
    finish_reduction(r, B, partials, g.counters + B.s, res + (long long)B.s * rstride);
}

struct TermDot {
    const double* x;
    const double* y;
    __device__ double operator()(int, long long i, double a) const { return fma(x[i], y[i], a); }
};
struct TermSum {
    const double* x;
    __device__ double operator()(int, long long i, double a) const { return a + x[i]; }
};
struct TermWsq {
    const double* x;
    const double* w;
    __device__ double operator()(int, long long i, double a) const
    {
        double r = x[i] * w[i];
        return fma(r, r, a);
    }
};
struct TermMgs {
    double* w;
    const double* vi;
    const double* h;
    int hstride;
    const double* vn;
    __device__ double operator()(int s, long long i, double a) const
    {
        double wn = fma(-h[(long long)s * hstride], vi[i], w[i]);
        w[i] = wn;
        return fma(wn, vn ? vn[i] : wn, a);
    }
};
struct TermScaleWsq {
    const double* w;
    const double* ih;
    int stride;
    double* v;
    const double* winv;
    __device__ double operator()(int s, long long i, double a) const
    {
        double vv = w[i] * ih[(long long)s * stride];
        v[i] = vv;
        double r = vv * winv[i];
        return fma(r, r, a);
    }
};
template <class Term>
static void run_reduce(const Term& t, const SegInfo& g, double* res, int rstride, double* partials,
                       cudaStream_t s)
{
    count();
    k_reduce<<<g.nblocks, kRedThreads, 0, s>>>(t, g, partials, res, rstride);
}

void launch_dot(const double* x, const double* y, const SegInfo& g, double* res, int rstride,
                double* partials, cudaStream_t s)
{
    run_reduce(TermDot{x, y}, g, res, rstride, partials, s);
}
void launch_vsum(const double* x, const SegInfo& g, double* res, int rstride, double* partials,
                 cudaStream_t s)
{
    run_reduce(TermSum{x}, g, res, rstride, partials, s);
}
void launch_wsq(const double* x, const double* winv, const SegInfo& g, double* res, int rstride,
                double* partials, cudaStream_t s)
{
    run_reduce(TermWsq{x, winv}, g, res, rstride, partials, s);
}
void launch_mgs(double* w, const double* vi, const double* h, int hstride, const double* vnext,
                const SegInfo& g, double* res, int rstride, double* partials, cudaStream_t s)
{
    run_reduce(TermMgs{w, vi, h, hstride, vnext}, g, res, rstride, partials, s);
}

// per segment: h = sqrt(hsq) (stored as H(j+1,j)) and its reciprocal, once
__global__ void k_store_sqrt(const double* hsq, double* hn, double* ih, int stride, int nseg,
                             const int* active)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg || (active && !active[s])) return;
    const long long o = (long long)s * stride;
    double h = sqrt(hsq[o]);
    hn[o] = h;
    ih[o] = 1.0 / h;
}

void launch_scale_wsq(const double* w, const double* hsq, double* hn, double* ih, int stride,
                      double* v, const double* winv, const SegInfo& g, double* res, double* partials,
                      cudaStream_t s)
{
    count();
    k_store_sqrt<<<(g.nseg + 127) / 128, 128, 0, s>>>(hsq, hn, ih, stride, g.nseg, g.active);
    run_reduce(TermScaleWsq{w, ih, stride, v, winv}, g, res, stride, partials, s);
}

// ---- fused Gram-Schmidt block of one Arnoldi step -----------------------------
// One cooperative launch does what the dot, the j+1 MGS passes, the square
// root and the scaling do as separate launches: pass p over every chunk of
// every active segment, a grid barrier, and so on.  Each chunk's partial sum
// and each segment's total are formed exactly as in k_reduce (same thread
// mapping, same trees), so the results are the same bits; every CTA forms
// the totals it needs from the previous pass's partials itself (partials
// alternate between two buffers, so no extra barrier is needed).
static constexpr long long kGridSpinLimit = 1LL << 22;

__device__ __forceinline__ SegBlock seg_block_at(const SegInfo& g, int b)
{
    SegBlock r;
    if (g.start) {
        r.s = g.blkseg[b];
        r.lo = g.start[r.s];
        r.hi = g.start[r.s + 1];
        r.b0 = g.block0[r.s];
        r.nb = g.block0[r.s + 1] - r.b0;
        r.lb = b - r.b0;
    } else {
        r.s = 0;
        r.lo = 0;
        r.hi = g.n1;
        r.b0 = 0;
        r.nb = g.nblocks;
        r.lb = b;
    }
    return r;
}

// grid-wide barrier with a bounded wait; false (and *err set) if it expired
__device__ __forceinline__ bool grid_barrier(unsigned int* count, unsigned int* gen, unsigned int nblk, int* err)
{
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok_s = 1;
        volatile unsigned int* vg = gen;
        const unsigned int g0 = *vg;
        __threadfence();
        if (atomicAdd(count, 1u) == nblk - 1) {
            // every CTA has arrived, and none arrives at the next barrier
            // before the generation moves: a plain store resets the count
            *reinterpret_cast<volatile unsigned int*>(count) = 0u;
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            long long it = 0;
            while (*vg == g0) {
                if (++it > kGridSpinLimit) {
                    atomicOr(err, 1);
                    ok_s = 0;
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok_s != 0;
}

template <class Term>
__device__ __forceinline__ double chunk_partial(const Term& term, const SegBlock& B, double* ws)
{
    const long long base = B.lo + (long long)B.lb * kRedChunk + threadIdx.x;
    double a = 0.0;
#pragma unroll 4
    for (int q = 0; q < kRedChunk / kRedThreads; ++q) {
        const long long i = base + (long long)q * kRedThreads;
        if (i < B.hi) a = term(B.s, i, a);
    }
    return block_sum_256(a, ws);
}

// the segment's total from its chunk partials (as the last block of
// k_reduce forms it), broadcast to every thread
__device__ __forceinline__ double segment_total(const SegBlock& B, const double* partials, double* ws, double* bc)
{
    double a = 0.0;
    for (int i = threadIdx.x; i < B.nb; i += kRedThreads) a = a + __ldcg(partials + B.b0 + i);
    const double t = block_sum_256(a, ws);
    if (threadIdx.x == 0) *bc = t;
    __syncthreads();
    const double r = *bc;
    __syncthreads();
    return r;
}

// CLUSTER: the grid is one thread-block cluster (at most 16 CTAs) and the
// passes are separated by the hardware cluster barrier; otherwise by the
// bounded global-memory barrier of a cooperative launch.
template <bool CLUSTER>
__global__ void __launch_bounds__(kRedThreads) k_gs_fused(SegInfo g, GsArgs A)
{
    __shared__ double ws[8];
    __shared__ double bc;
    const int j = A.j;
    for (int p = 0; p <= j + 2; ++p) {
        double* part = A.partials + (size_t)(p & 1) * A.pstride;
        const double* prev = A.partials + (size_t)((p + 1) & 1) * A.pstride;
        int cs = -1;          // segment whose previous-pass total is cached
        double ch = 0.0;
        for (int b = blockIdx.x; b < g.nblocks; b += gridDim.x) {
            const SegBlock B = seg_block_at(g, b);
            if (g.active && !g.active[B.s]) continue;
            const long long so = (long long)B.s * A.stride;
            double r;
            if (p == 0) {
                r = chunk_partial(TermDot{A.w, A.V}, B, ws);
            } else {
                if (B.s != cs) {
                    ch = segment_total(B, prev, ws, &bc);     // total of pass p-1
                    cs = B.s;
                }
                const double h = ch;
                const bool writer = (b == B.b0) && threadIdx.x == 0;
                if (p <= j + 1) {
                    // h = H(p-1, j); w -= h v_{p-1}; dot with v_p (or with w after the last)
                    if (writer) A.Hc[so + p - 1] = h;
                    double* hp = &bc;     // TermMgs reads h through a pointer
                    (void)hp;
                    const double* vi = A.V + (size_t)(p - 1) * A.ldV;
                    const double* vn = (p <= j) ? A.V + (size_t)p * A.ldV : nullptr;
                    struct {
                        double* w;
                        const double* vi;
                        double h;
                        const double* vn;
                        __device__ double operator()(int, long long i, double a) const
                        {
                            double wn = fma(-h, vi[i], w[i]);
                            w[i] = wn;
                            return fma(wn, vn ? vn[i] : wn, a);
                        }
                    } t{A.w, vi, h, vn};
                    r = chunk_partial(t, B, ws);
                } else {
                    // h = ||w||^2: H(j+1, j) = sqrt, v_{j+1} = w / H(j+1, j), weighted norm
                    const double hn = sqrt(h);
                    const double ih = 1.0 / hn;
                    if (writer) {
                        A.hsq[so] = h;
                        A.Hc[so + j + 1] = hn;
                        A.ih[so] = ih;
                    }
                    double* v = A.V + (size_t)(j + 1) * A.ldV;
                    struct {
                        const double* w;
                        double ih;
                        double* v;
                        const double* winv;
                        __device__ double operator()(int, long long i, double a) const
                        {
                            double vv = w[i] * ih;
                            v[i] = vv;
                            double rr = vv * winv[i];
                            return fma(rr, rr, a);
                        }
                    } t{A.w, ih, v, A.winv};
                    r = chunk_partial(t, B, ws);
                }
            }
            if (threadIdx.x == 0) part[b] = r;
        }
        if (CLUSTER) {
            __threadfence();
            asm volatile("barrier.cluster.arrive.release.aligned;\n"
                         "barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
        } else if (!grid_barrier(A.bar, A.bar + 1, gridDim.x, A.err)) {
            return;
        }
    }
    // the weighted norm of v_{j+1} (total of the last pass)
    const double* last = A.partials + (size_t)((j + 2) & 1) * A.pstride;
    for (int b = blockIdx.x; b < g.nblocks; b += gridDim.x) {
        const SegBlock B = seg_block_at(g, b);
        if (g.active && !g.active[B.s]) continue;
        if (b != B.b0) continue;
        const double sv = segment_total(B, last, ws, &bc);
        if (threadIdx.x == 0) A.sv[(long long)B.s * A.stride] = sv;
    }
}

// The Gram-Schmidt block for problems of at most 16 chunks (one thread-block
// cluster, one chunk per CTA).  The passes and their arithmetic are those of
// k_gs_fused, in the same order (same bits), but: each thread keeps its 32
// items of w in registers for the whole block and writes w back once; the
// basis vector of the next pass is loaded into registers before the barrier,
// so its latency overlaps the wait, and the current one sits in the thread's
// own slots of 64 KB of shared memory; the chunk partials go through distributed shared
// memory instead of global memory, and every warp forms the segment totals
// itself (at most 16 partials), so a pass costs one CTA barrier and one
// cluster barrier.  Every CTA executes every cluster barrier, including a
// last one after the final reads of its peers' shared memory.
__global__ void __launch_bounds__(kRedThreads, 1) k_gs_cluster(SegInfo g, GsArgs A)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    constexpr int Q = kRedChunk / kRedThreads;      // items per thread
    __shared__ double ws[8];
    __shared__ double mypart[2];                    // chunk partial, by pass parity
    extern __shared__ double vsm[];                 // [Q][kRedThreads]: basis vector of this pass
    double* vc = vsm + threadIdx.x;                 // item q of this thread at vc[q * kRedThreads]
    const int j = A.j;
    const int b = (int)blockIdx.x;                  // chunk = cluster rank
    const int lane = threadIdx.x & 31;
    const SegBlock B = seg_block_at(g, b);
    const bool act = !(g.active && !g.active[B.s]);
    const long long base = B.lo + (long long)B.lb * kRedChunk + threadIdx.x;
    const long long so = (long long)B.s * A.stride;
    const bool writer = (b == B.b0) && threadIdx.x == 0;
    double w[Q], vn[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const long long i = base + (long long)q * kRedThreads;
        const bool in = act && i < B.hi;
        w[q] = in ? A.w[i] : 0.0;
        vc[q * kRedThreads] = in ? A.V[i] : 0.0;
        vn[q] = (in && j >= 1) ? A.V[(size_t)A.ldV + i] : 0.0;
    }
    // total of the previous pass's chunk partials of this chunk's segment,
    // formed as segment_total forms it (thread t: 0 + P[t]; block tree with
    // the seven all-zero warps)
    auto seg_total = [&](int par) -> double {
        double a = 0.0;
        if (lane < B.nb) a = 0.0 + *cl.map_shared_rank(&mypart[par], (unsigned)(B.b0 + lane));
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) a = a + __shfl_xor_sync(0xffffffffu, a, d);
        const double z = 0.0;
        return ((a + z) + (z + z)) + ((z + z) + (z + z));
    };
    for (int p = 0; p <= j + 2; ++p) {
        double a = 0.0;
        if (p == 0) {
#pragma unroll
            for (int q = 0; q < Q; ++q)
                if (base + (long long)q * kRedThreads < B.hi) a = fma(w[q], vc[q * kRedThreads], a);
        } else {
            const double h = seg_total((p + 1) & 1);
            if (p <= j + 1) {
                // h = H(p-1, j); w -= h v_{p-1}; dot with v_p (or with w after the last)
                if (writer && act) A.Hc[so + p - 1] = h;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    if (base + (long long)q * kRedThreads >= B.hi) continue;
                    const double wn = fma(-h, vc[q * kRedThreads], w[q]);
                    w[q] = wn;
                    a = fma(wn, (p <= j) ? vn[q] : wn, a);
                }
            } else {
                // h = ||w||^2: H(j+1, j) = sqrt, v_{j+1} = w / H(j+1, j), weighted norm
                const double hn = sqrt(h);
                const double ih = 1.0 / hn;
                if (writer && act) {
                    A.hsq[so] = h;
                    A.Hc[so + j + 1] = hn;
                    A.ih[so] = ih;
                }
                double* v = A.V + (size_t)(j + 1) * A.ldV;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    const long long i = base + (long long)q * kRedThreads;
                    if (!act || i >= B.hi) continue;
                    const double vv = w[q] * ih;
                    v[i] = vv;
                    const double rr = vv * vn[q];        // vn holds winv here
                    a = fma(rr, rr, a);
                }
            }
        }
        const double r = block_sum_256(a, ws);
        if (threadIdx.x == 0) mypart[p & 1] = r;
        if (p >= 1) {
            // the next pass's vector: v_{p+1}, or the weights for the scaling pass
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const long long i = base + (long long)q * kRedThreads;
                const bool in = act && i < B.hi;
                vc[q * kRedThreads] = vn[q];
                if (p + 1 <= j) vn[q] = in ? A.V[(size_t)(p + 1) * A.ldV + i] : 0.0;
                else if (p + 1 == j + 2) vn[q] = in ? A.winv[i] : 0.0;
            }
        }
        cl.sync();
    }
    // the weighted norm of v_{j+1} (total of the last pass): every lane of
    // warp 0 takes part in the warp shuffles, lane 0 stores; then w
    if (b == B.b0 && act && (threadIdx.x >> 5) == 0) {
        const double sv = seg_total((j + 2) & 1);
        if (threadIdx.x == 0) A.sv[so] = sv;
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const long long i = base + (long long)q * kRedThreads;
        if (act && i < B.hi) A.w[i] = w[q];
    }
    cl.sync();        // peers may still read this CTA's partials
}

// The Gram-Schmidt block for problems of at most 16 chunks, spread over the
// GPU.  One pass of a chunk is 8,192 items x 2 FP64 fused multiply-adds;
// with one CTA per chunk it runs on one SM, whose FP64 pipe issues one
// warp instruction per 16 cycles (about 4 us a pass).  Here each of the
// chunk's eight warps is a CTA of its own (up to 128 CTAs, one warp per
// SM): thread l of CTA 8b + v plays thread 32v + l of chunk b in k_gs_fused
// (same items, same chains), the warp's butterfly sum goes to global
// memory, and after the bounded grid barrier every CTA forms the chunk
// partials (the eight-warp tree of block_sum_256) and the segment total
// (as segment_total forms it) itself -- the same bits.  w and the next
// basis vector stay in registers, the current one in shared memory.
template <int WPC>
__global__ void __launch_bounds__(32 * WPC, 1) k_gs_warps(SegInfo g, GsArgs A)
{
    constexpr int Q = kRedChunk / kRedThreads;      // items per thread
    constexpr int NT = 32 * WPC;                    // threads per CTA
    __shared__ double vcs[Q * NT];                  // current basis vector, [q][thread]
    const int j = A.j;
    const int cpb = 8 / WPC;                        // CTAs per chunk
    const int b = (int)(blockIdx.x / (unsigned)cpb);
    const int wv = (int)(blockIdx.x % (unsigned)cpb) * WPC + (int)(threadIdx.x >> 5);   // warp of the chunk
    const int lane = threadIdx.x & 31;
    const int tix = threadIdx.x;
    const SegBlock B = seg_block_at(g, b);
    const bool act = !(g.active && !g.active[B.s]);
    const long long base = B.lo + (long long)B.lb * kRedChunk + wv * 32 + lane;
    const long long so = (long long)B.s * A.stride;
    const bool writer = (b == B.b0) && wv == 0 && lane == 0;
    double w[Q], vn[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const long long i = base + (long long)q * kRedThreads;
        const bool in = act && i < B.hi;
        w[q] = in ? A.w[i] : 0.0;
        vcs[q * NT + tix] = in ? A.V[i] : 0.0;
        vn[q] = (in && j >= 1) ? A.V[(size_t)A.ldV + i] : 0.0;
    }
    // total of the previous pass over this chunk's segment: chunk partials
    // from their eight warp sums, then lane c holds 0 + P[c] and the block
    // tree with the seven all-zero warps follows
    auto seg_total = [&](int par) -> double {
        const double* P = A.wpart + (size_t)par * 128;
        double a = 0.0;
        if (lane < B.nb) {
            const double* c = P + (size_t)(B.b0 + lane) * 8;
            const double cp = ((__ldcg(c) + __ldcg(c + 1)) + (__ldcg(c + 2) + __ldcg(c + 3))) +
                              ((__ldcg(c + 4) + __ldcg(c + 5)) + (__ldcg(c + 6) + __ldcg(c + 7)));
            a = 0.0 + cp;
        }
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) a = a + __shfl_xor_sync(0xffffffffu, a, d);
        const double z = 0.0;
        return ((a + z) + (z + z)) + ((z + z) + (z + z));
    };
    for (int p = 0; p <= j + 2; ++p) {
        double a = 0.0;
        if (p == 0) {
#pragma unroll
            for (int q = 0; q < Q; ++q)
                if (base + (long long)q * kRedThreads < B.hi) a = fma(w[q], vcs[q * NT + tix], a);
        } else {
            const double h = seg_total((p + 1) & 1);
            if (p <= j + 1) {
                // h = H(p-1, j); w -= h v_{p-1}; dot with v_p (or with w after the last)
                if (writer && act) A.Hc[so + p - 1] = h;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    if (base + (long long)q * kRedThreads >= B.hi) continue;
                    const double wn = fma(-h, vcs[q * NT + tix], w[q]);
                    w[q] = wn;
                    a = fma(wn, (p <= j) ? vn[q] : wn, a);
                }
            } else {
                // h = ||w||^2: H(j+1, j) = sqrt, v_{j+1} = w / H(j+1, j), weighted norm
                const double hn = sqrt(h);
                const double ih = 1.0 / hn;
                if (writer && act) {
                    A.hsq[so] = h;
                    A.Hc[so + j + 1] = hn;
                    A.ih[so] = ih;
                }
                double* v = A.V + (size_t)(j + 1) * A.ldV;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    const long long i = base + (long long)q * kRedThreads;
                    if (!act || i >= B.hi) continue;
                    const double vv = w[q] * ih;
                    v[i] = vv;
                    const double rr = vv * vn[q];        // vn holds winv here
                    a = fma(rr, rr, a);
                }
            }
        }
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) a = a + __shfl_xor_sync(0xffffffffu, a, d);
        if (lane == 0) A.wpart[(size_t)(p & 1) * 128 + (size_t)b * 8 + wv] = a;
        if (p >= 1) {
            // the next pass's vector: v_{p+1}, or the weights for the scaling pass
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const long long i = base + (long long)q * kRedThreads;
                const bool in = act && i < B.hi;
                vcs[q * NT + tix] = vn[q];
                if (p + 1 <= j) vn[q] = in ? A.V[(size_t)(p + 1) * A.ldV + i] : 0.0;
                else if (p + 1 == j + 2) vn[q] = in ? A.winv[i] : 0.0;
            }
        }
        if (!grid_barrier(A.bar, A.bar + 1, gridDim.x, A.err)) return;
    }
    // the weighted norm of v_{j+1} (total of the last pass), then w
    if (b == B.b0 && wv == 0 && act) {             // warp 0 of the chunk, all its lanes
        const double sv = seg_total((j + 2) & 1);
        if (lane == 0) A.sv[so] = sv;
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const long long i = base + (long long)q * kRedThreads;
        if (act && i < B.hi) A.w[i] = w[q];
    }
}

// Failure-path probe of the bounded grid barrier: CTA 1 leaves without
// arriving, so CTA 0's wait must run out and raise *err.
__global__ void k_barrier_probe(unsigned int* bar, int* err)
{
    if (blockIdx.x == 1) return;
    grid_barrier(bar, bar + 1, 2u, err);
}

int barrier_probe(int* timed_out)
{
    unsigned int* bar = nullptr;
    int* err = nullptr;
    if (cudaMalloc(&bar, 2 * sizeof(unsigned int)) != cudaSuccess) return 1;
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) {
        cudaFree(bar);
        return 1;
    }
    cudaMemset(bar, 0, 2 * sizeof(unsigned int));
    cudaMemset(err, 0, sizeof(int));
    k_barrier_probe<<<2, 32>>>(bar, err);
    cudaError_t e = cudaDeviceSynchronize();
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(bar);
    cudaFree(err);
    if (e != cudaSuccess) return 1;
    *timed_out = h;
    return 0;
}

static int g_nsm = 0;       // SMs of the device (set with the Gram-Schmidt launch shape)
// warps of a chunk per CTA of the warp-spread Gram-Schmidt kernel (1, 2, 4
// or 8): fewer CTAs make the grid barrier cheaper, more warps per SM make
// the FP64 pipe the limit
static constexpr int kGsWarpsPerCta = 1;
static constexpr int kGsMaxCluster = 16;
static constexpr int kGsClusterSmem = kRedChunk * (int)sizeof(double);   // one chunk of a vector
static int g_gs_cluster_max = 0;    // largest cluster the device schedules for the cluster kernel

int gs_fused_grid(int nsm)
{
    g_nsm = nsm;
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_gs_fused<false>, kRedThreads, 0) != cudaSuccess)
        return 0;
    // clusters of more than 8 CTAs are a non-portable size: use them only if
    // the device can schedule one
    g_gs_cluster_max = 0;
    if (cudaFuncSetAttribute(k_gs_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        cudaGetLastError();
    if (cudaFuncSetAttribute(k_gs_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, kGsClusterSmem) !=
        cudaSuccess)
        return occ * nsm;       // no cluster variant
    for (int cs : {kGsMaxCluster, 8}) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)cs);
        cfg.blockDim = dim3(kRedThreads);
        cfg.dynamicSmemBytes = kGsClusterSmem;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int nc = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, k_gs_cluster, &cfg) == cudaSuccess && nc > 0) {
            g_gs_cluster_max = cs;
            break;
        }
        cudaGetLastError();
    }
    return occ * nsm;
}

// problems of at most 16 chunks take the warp-spread kernel when the caller
// passes its warp-sum buffer (wpart), the one-cluster kernel otherwise
static bool gs_use_warps(const SegInfo& g, int max_grid, bool warps)
{
    const int grid = std::min(g.nblocks, max_grid);
    return warps && grid == g.nblocks && g.nblocks <= 16;
}


// co-resident CTAs for nblocks chunks: as few rounds as max_grid allows, and
// the chunks spread evenly over them (no half-empty last round); which CTA
// forms a chunk's partial does not change it
static int balanced_grid(int nblocks, int max_grid)
{
    if (nblocks <= max_grid || max_grid < 1) return std::min(nblocks, std::max(max_grid, 1));
    const int rounds = (nblocks + max_grid - 1) / max_grid;
    return (nblocks + rounds - 1) / rounds;
}

cudaError_t launch_gs_fused(const SegInfo& g, const GsArgs& A, int max_grid, cudaStream_t s)
{
    count();
    cudaLaunchConfig_t cfg = {};
    const int grid = balanced_grid(g.nblocks, max_grid);
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kRedThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (gs_use_warps(g, max_grid, A.wpart != nullptr)) {
        // kGsWarpsPerCta warps of a chunk per CTA, cooperative
        cfg.gridDim = dim3((unsigned)(8 / kGsWarpsPerCta * g.nblocks));
        cfg.blockDim = dim3(32 * kGsWarpsPerCta);
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        return cudaLaunchKernelEx(&cfg, k_gs_warps<kGsWarpsPerCta>, g, A);
    }
    if (grid <= g_gs_cluster_max && grid == g.nblocks) {
        // one chunk per CTA, the whole grid one cluster
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)grid;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.dynamicSmemBytes = kGsClusterSmem;
        return cudaLaunchKernelEx(&cfg, k_gs_cluster, g, A);
    }
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    return cudaLaunchKernelEx(&cfg, k_gs_fused<false>, g, A);
}

// ---- classical Gram-Schmidt twice (CGS2), fused --------------------------------
// The Gram-Schmidt block of an Arnoldi step as two classical passes:
//   pass 0: c_q = <w, v_q> for every q <= j at once
//   pass 1: w -= sum_q c_q v_q (q ascending, one FMA each); d_q = <w, v_q>
//   pass 2: w -= sum_q d_q v_q; H(q, j) = c_q + d_q; <w, w>
//   pass 3: H(j+1, j) = sqrt, v_{j+1} = w / H(j+1, j), weighted norm
// Every dot is formed as k_reduce forms one (same thread mapping, same
// trees, same segment totals), so each equals a separate fixed-order
// reduction bit for bit.  Four grid-wide (or cluster-wide) barriers per
// Arnoldi step instead of j+3, and 3j+10 vector passes of memory traffic
// instead of 4j+8.  Items are taken one at a time (the thread's 32 items
// of the chunk in ascending order) with the j+1 running dot sums in
// registers (NV >= j+1 of them, a multiple of 8), so pass 1 reads each
// basis entry from memory once and again at once from L1.  The partials of
// the j+1 dots of a pass sit at partials + parity * parstride + q * pstride
// + chunk.  Dynamic shared memory: 9 NV doubles (warp sums and totals).
constexpr int kCgs2MaxNV = 64;

template <bool CLUSTER, int NV>
__global__ void __launch_bounds__(kRedThreads) k_gs_cgs2(SegInfo g, GsArgs A)
{
    constexpr int Q = kRedChunk / kRedThreads;
    extern __shared__ double sm2[];
    const int j = A.j;
    const int nv = j + 1;
    double* ws = sm2;                 // [NV][8] warp sums
    double* tot = sm2 + 8 * NV;       // [NV] segment totals of the previous pass
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    auto warp_put = [&](int q, double a) {
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) a = a + __shfl_xor_sync(0xffffffffu, a, d);
        if (lane == 0) ws[8 * q + warp] = a;
    };
    // the chunk partials of n values: the eight warps' tree on thread q
    auto emit = [&](int n, double* part, int b) {
        __syncthreads();
        if ((int)threadIdx.x < n) {
            const double* s = ws + 8 * threadIdx.x;
            part[(size_t)threadIdx.x * A.pstride + b] = ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
        }
        __syncthreads();
    };
    for (int p = 0; p <= 3; ++p) {
        double* part = A.partials + (size_t)(p & 1) * A.parstride;
        const double* prev = A.partials + (size_t)((p + 1) & 1) * A.parstride;
        const int ntot = (p == 0) ? 0 : (p <= 2 ? nv : 1);     // values of the previous pass
        int cs = -1;
        for (int b = blockIdx.x; b < g.nblocks; b += gridDim.x) {
            const SegBlock B = seg_block_at(g, b);
            if (g.active && !g.active[B.s]) continue;
            const long long so = (long long)B.s * A.stride;
            const bool writer = (b == B.b0) && threadIdx.x == 0;
            if (ntot > 0 && B.s != cs) {
                // totals of the previous pass for this segment (segment_total's order)
                for (int q = 0; q < ntot; ++q) {
                    double a = 0.0;
                    for (int i = threadIdx.x; i < B.nb; i += kRedThreads)
                        a = a + __ldcg(prev + (size_t)q * A.pstride + B.b0 + i);
                    warp_put(q, a);
                }
                __syncthreads();
                if ((int)threadIdx.x < ntot) {
                    const double* s = ws + 8 * threadIdx.x;
                    tot[threadIdx.x] = ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
                }
                __syncthreads();
                cs = B.s;
            }
            const long long base = B.lo + (long long)B.lb * kRedChunk + threadIdx.x;
            // items in groups of KG (ascending), so that KG loads of every
            // basis vector are in flight at once; per value the sums still
            // run over the items in ascending order
            constexpr int KG = 4;
            if (p <= 1) {
                if (p == 1 && writer)
                    for (int q = 0; q < nv; ++q) A.Hc[so + q] = tot[q];
                double acc[NV];
#pragma unroll
                for (int q = 0; q < NV; ++q) acc[q] = 0.0;
                for (int k0 = 0; k0 < Q; k0 += KG) {
                    if (base + (long long)k0 * kRedThreads >= B.hi) break;
                    long long ii[KG];
                    bool in[KG];
                    double y[KG];
#pragma unroll
                    for (int u = 0; u < KG; ++u) {
                        ii[u] = base + (long long)(k0 + u) * kRedThreads;
                        in[u] = ii[u] < B.hi;
                        y[u] = in[u] ? A.w[ii[u]] : 0.0;
                    }
                    if (p == 1) {
                        // w -= sum_q c_q v_q, q ascending
#pragma unroll
                        for (int q = 0; q < NV; ++q) {
                            if (q >= nv) break;
                            const double h = tot[q];
                            const double* vq = A.V + (size_t)q * A.ldV;
#pragma unroll
                            for (int u = 0; u < KG; ++u)
                                if (in[u]) y[u] = fma(-h, vq[ii[u]], y[u]);
                        }
#pragma unroll
                        for (int u = 0; u < KG; ++u)
                            if (in[u]) A.w[ii[u]] = y[u];
                    }
#pragma unroll
                    for (int q = 0; q < NV; ++q) {
                        if (q >= nv) break;
                        const double* vq = A.V + (size_t)q * A.ldV;
#pragma unroll
                        for (int u = 0; u < KG; ++u)
                            if (in[u]) acc[q] = fma(y[u], vq[ii[u]], acc[q]);
                    }
                }
#pragma unroll
                for (int q = 0; q < NV; ++q)
                    if (q < nv) warp_put(q, acc[q]);
                emit(nv, part, b);
            } else if (p == 2) {
                // w -= sum_q d_q v_q; H(q, j) = c_q + d_q; <w, w>
                if (writer)
                    for (int q = 0; q < nv; ++q) A.Hc[so + q] = A.Hc[so + q] + tot[q];
                double a = 0.0;
                for (int k0 = 0; k0 < Q; k0 += KG) {
                    if (base + (long long)k0 * kRedThreads >= B.hi) break;
                    long long ii[KG];
                    bool in[KG];
                    double y[KG];
#pragma unroll
                    for (int u = 0; u < KG; ++u) {
                        ii[u] = base + (long long)(k0 + u) * kRedThreads;
                        in[u] = ii[u] < B.hi;
                        y[u] = in[u] ? A.w[ii[u]] : 0.0;
                    }
#pragma unroll
                    for (int q = 0; q < NV; ++q) {
                        if (q >= nv) break;
                        const double h = tot[q];
                        const double* vq = A.V + (size_t)q * A.ldV;
#pragma unroll
                        for (int u = 0; u < KG; ++u)
                            if (in[u]) y[u] = fma(-h, vq[ii[u]], y[u]);
                    }
#pragma unroll
                    for (int u = 0; u < KG; ++u)
                        if (in[u]) {
                            A.w[ii[u]] = y[u];
                            a = fma(y[u], y[u], a);
                        }
                }
                warp_put(0, a);
                emit(1, part, b);
            } else {
                // H(j+1, j) = sqrt(<w, w>), v_{j+1} = w / H(j+1, j), weighted norm
                const double h = tot[0];
                const double hn = sqrt(h);
                const double ih = 1.0 / hn;
                if (writer) {
                    A.hsq[so] = h;
                    A.Hc[so + j + 1] = hn;
                    A.ih[so] = ih;
                }
                double* v = A.V + (size_t)(j + 1) * A.ldV;
                double a = 0.0;
#pragma unroll 8
                for (int k = 0; k < Q; ++k) {
                    const long long i = base + (long long)k * kRedThreads;
                    if (i < B.hi) {
                        const double vv = A.w[i] * ih;
                        v[i] = vv;
                        const double rr = vv * A.winv[i];
                        a = fma(rr, rr, a);
                    }
                }
                warp_put(0, a);
                emit(1, part, b);
            }
        }
        if (CLUSTER) {
            __threadfence();
            asm volatile("barrier.cluster.arrive.release.aligned;\n"
                         "barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
        } else if (!grid_barrier(A.bar, A.bar + 1, gridDim.x, A.err)) {
            return;
        }
    }
    // the weighted norm of v_{j+1} (total of the last pass)
    __shared__ double ws8[8];
    __shared__ double bc;
    const double* last = A.partials + (size_t)(3 & 1) * A.parstride;
    for (int b = blockIdx.x; b < g.nblocks; b += gridDim.x) {
        const SegBlock B = seg_block_at(g, b);
        if (g.active && !g.active[B.s]) continue;
        if (b != B.b0) continue;
        const double sv = segment_total(B, last, ws8, &bc);
        if (threadIdx.x == 0) A.sv[(long long)B.s * A.stride] = sv;
    }
}

namespace {
using Cgs2Kernel = void (*)(SegInfo, GsArgs);
template <bool CLUSTER>
Cgs2Kernel cgs2_kernel(int nv)
{
    switch ((nv + 7) / 8) {
    case 1: return k_gs_cgs2<CLUSTER, 8>;
    case 2: return k_gs_cgs2<CLUSTER, 16>;
    case 3: return k_gs_cgs2<CLUSTER, 24>;
    case 4: return k_gs_cgs2<CLUSTER, 32>;
    case 5: return k_gs_cgs2<CLUSTER, 40>;
    case 6: return k_gs_cgs2<CLUSTER, 48>;
    case 7: return k_gs_cgs2<CLUSTER, 56>;
    case 8: return k_gs_cgs2<CLUSTER, 64>;
    default: return nullptr;
    }
}
size_t cgs2_smem(int nv) { return sizeof(double) * 9 * (size_t)(((nv + 7) / 8) * 8); }
int g_cgs2_cluster_ok = 0;
int g_cgs2_occ[kCgs2MaxNV / 8] = {};     // co-resident CTAs per SM, by basis-size bucket
}  // namespace

int gs_cgs2_max_dim() { return kCgs2MaxNV - 1; }

// occupancy of every instantiation up to maxk + 1 basis vectors; nsm if all
// of them can be launched cooperatively, 0 otherwise
int gs_cgs2_grid(int nsm, int maxk)
{
    if (maxk + 1 > kCgs2MaxNV) return 0;
    const int nb = (maxk + 1 + 7) / 8;
    for (int k = 0; k < nb; ++k) {
        const int nv = 8 * (k + 1);
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, cgs2_kernel<false>(nv), kRedThreads,
                                                          cgs2_smem(nv)) != cudaSuccess || occ < 1) {
            cudaGetLastError();
            return 0;
        }
        g_cgs2_occ[k] = occ;
    }
    g_cgs2_cluster_ok = 0;
    if (g_gs_cluster_max > 0) {
        // every instantiation must schedule a cluster of the largest size used
        bool ok = true;
        for (int k = 0; k < nb && ok; ++k) {
            const int nv = 8 * (k + 1);
            if (cudaFuncSetAttribute(cgs2_kernel<true>(nv), cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                cudaSuccess) {
                cudaGetLastError();
                ok = false;
                break;
            }
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)g_gs_cluster_max);
            cfg.blockDim = dim3(kRedThreads);
            cfg.dynamicSmemBytes = cgs2_smem(nv);
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = (unsigned)g_gs_cluster_max;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int ncl = 0;
            if (cudaOccupancyMaxActiveClusters(&ncl, cgs2_kernel<true>(nv), &cfg) != cudaSuccess || ncl < 1) {
                cudaGetLastError();
                ok = false;
            }
        }
        g_cgs2_cluster_ok = ok ? 1 : 0;
    }
    return nsm;
}

cudaError_t launch_gs_cgs2(const SegInfo& g, const GsArgs& A, int nsm, cudaStream_t s)
{
    count();
    const int nv = A.j + 1;
    if (nv > kCgs2MaxNV || g_cgs2_occ[(nv - 1) / 8] < 1) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg = {};
    const int grid = balanced_grid(g.nblocks, g_cgs2_occ[(nv - 1) / 8] * nsm);
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kRedThreads);
    cfg.dynamicSmemBytes = cgs2_smem(nv);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (g_cgs2_cluster_ok && grid <= g_gs_cluster_max && grid == g.nblocks) {
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)grid;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        return cudaLaunchKernelEx(&cfg, cgs2_kernel<true>(nv), g, A);
    }
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    return cudaLaunchKernelEx(&cfg, cgs2_kernel<false>(nv), g, A);
}

// ---- elementwise, over segments (same block mapping as the reductions) -------
template <class Op>
__global__ void __launch_bounds__(kRedThreads) k_segmap(Op op, SegInfo g)
{
    const SegBlock B = seg_block(g);
    if (g.active && !g.active[B.s]) return;
    const long long base = B.lo + (long long)B.lb * kRedChunk + threadIdx.x;
#pragma unroll 4
    for (int q = 0; q < kRedChunk / kRedThreads; ++q) {
        const long long i = base + (long long)q * kRedThreads;
        if (i < B.hi) op(B.s, i);
    }
}

// The same elementwise work on a finer grid: block b covers part b % sub of
// chunk b / sub (kRedChunk / sub items).  Elementwise results do not depend
// on the mapping, so small problems (few chunks) spread over the whole GPU.
template <class Op>
__global__ void __launch_bounds__(kRedThreads) k_segmap_sub(Op op, SegInfo g, int sub)
{
    const SegBlock B = seg_block_at(g, (int)(blockIdx.x / (unsigned)sub));
    if (g.active && !g.active[B.s]) return;
    const int per = kRedChunk / sub;
    const long long base =
        B.lo + (long long)B.lb * kRedChunk + (long long)(blockIdx.x % (unsigned)sub) * per + threadIdx.x;
    for (int q = 0; q < per / kRedThreads; ++q) {
        const long long i = base + (long long)q * kRedThreads;
        if (i < B.hi) op(B.s, i);
    }
}

// chunk parts per block: the smallest power of two (at most 32) that gives
// four blocks per SM, 1 for large problems
template <class Op>
static void segmap_launch(const Op& op, const SegInfo& g, cudaStream_t s)
{
    int sub = 1;
    while (sub < kRedChunk / kRedThreads && (long long)g.nblocks * sub < 4LL * (g_nsm > 0 ? g_nsm : 152)) sub *= 2;
    count();
    if (sub == 1)
        k_segmap<<<g.nblocks, kRedThreads, 0, s>>>(op, g);
    else
        k_segmap_sub<<<g.nblocks * sub, kRedThreads, 0, s>>>(op, g, sub);
}

struct OpScale {
    const double* x;
    const double* a;
    int astride;
    double* y;
    __device__ void operator()(int s, long long i) const { y[i] = x[i] * a[(long long)s * astride]; }
};
struct OpWinv {
    const double* u;
    double rtol, atol;
    double* w;
    __device__ void operator()(int, long long i) const { w[i] = 1.0 / fma(rtol, fabs(u[i]), atol); }
};
struct OpCombine {
    const double* u;
    const double* V;
    long long ldV;
    const double* c;
    int cstride;
    const int* m;
    double* out;
    __device__ void operator()(int s, long long i) const
    {
        const double* cs = c + (long long)s * cstride;
        const int ms = m[s];
        double a = u[i];
        for (int q = 0; q < ms; ++q) a = fma(cs[q], V[(long long)q * ldV + i], a);
        out[i] = a;
    }
};

struct OpCopy2 {
    const double* a;
    double* b;
    const double* c;
    double* d;
    __device__ void operator()(int, long long i) const
    {
        b[i] = a[i];
        d[i] = c[i];
    }
};

// D = (g1 - g0 - sum_q z_q V_q) dt/3, the local error of the step
struct OpErrD {
    const double* g1;
    const double* g0;
    const double* V;
    long long ldV;
    const double* z;
    int zstride;
    const int* mz;
    const double* dt3;
    int dstride;
    double* D;
    __device__ void operator()(int s, long long i) const
    {
        const double* zs = z + (long long)s * zstride;
        const int m = mz[s];
        double d = g1[i] - g0[i];
        for (int q = 0; q < m; ++q) d = fma(-zs[q], V[(long long)q * ldV + i], d);
        D[i] = d * dt3[(long long)s * dstride];
    }
};

void launch_seg_copy2(const double* a, double* b, const double* c, double* d, const SegInfo& g,
                      cudaStream_t s)
{
    segmap_launch(OpCopy2{a, b, c, d}, g, s);
}
void launch_seg_scale(const double* x, const double* a, int astride, double* y, const SegInfo& g,
                      cudaStream_t s)
{
    segmap_launch(OpScale{x, a, astride, y}, g, s);
}
void launch_winv(const double* u, double rtol, double atol, double* winv, const SegInfo& g,
                 cudaStream_t s)
{
    segmap_launch(OpWinv{u, rtol, atol, winv}, g, s);
}
void launch_combine(const double* u, const double* V, long long ldV, const double* c, int cstride,
                    const int* m, double* out, const SegInfo& g, cudaStream_t s)
{
    segmap_launch(OpCombine{u, V, ldV, c, cstride, m, out}, g, s);
}

// the step's error in two passes, as the oracle forms it: D elementwise
// (any grid), then the fixed-order weighted sum of squares of D
void launch_err(const double* g1, const double* g0, const double* V, long long ldV, const double* z,
                int zstride, const int* mz, const double* dt3, int dstride, const double* winv,
                const SegInfo& g, double* res, int rstride, double* partials, double* D, cudaStream_t s)
{
    segmap_launch(OpErrD{g1, g0, V, ldV, z, zstride, mz, dt3, dstride, D}, g, s);
    run_reduce(TermWsq{D, winv}, g, res, rstride, partials, s);
}

// ---- total water content --------------------------------------------------
// Terms are laid out scenario by scenario: [macro nodes of s | cells of s].
__device__ __forceinline__ long long water_slot_node(const MacroDev& M, int i)
{
    if (M.nscen <= 1) return i;
    const int s = i / M.scen_nodes;
    return (long long)s * (M.scen_nodes + M.scen_cells) + (i - s * M.scen_nodes);
}
__device__ __forceinline__ long long water_slot_cell(const MacroDev& M, int k)
{
    if (M.nscen <= 1) return (long long)M.Mn + k;
    const int s = k / M.scen_cells;
    return (long long)s * (M.scen_nodes + M.scen_cells) + M.scen_nodes + (k - s * M.scen_cells);
}

__global__ void k_water_macro(Problem P, const double* __restrict__ u, double* __restrict__ terms)
{
    const MacroDev& M = P.M;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.Mn) return;
    const VGPar& pA = M.scen_pA ? M.scen_pA[i / M.scen_nodes] : P.pA;
    double Se = vg_se(u[M.node_off ? M.node_off[i] : i], pA, &d_tables);
    terms[water_slot_node(M, i)] = (M.epsA * M.cv[i]) * fma(pA.dth, Se, pA.thr);
}

// one warp per cell; lane l sums nodes l, l+32, ... (the fixed lane order)
// The solution writer's calibration (src/save_solution.cpp:41-102): the
// micro-boundary entries of state x, which the kernels never evolve (the
// cells use the macro interpolant there), overwritten with the interpolant
// at centroid + s vectors (model_type 1: the centroid); one warp per cell,
// one lane per boundary node, the operation sequence of the host version
// (tsr_calibrate_micro_boundary) and of the cell kernel's boundary pass.
// Learned cells carry no micro nodes and are left alone.
__global__ void k_calibrate(Problem P, double* __restrict__ x)
{
    const MacroDev& M = P.M;
    const MicroSet& S = P.m;
    const int lane = threadIdx.x & 31;
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (k >= M.Ne) return;
    const int nv = M.nv, Ne = M.Ne;
    const TplDesc D = S.tpl[S.cell_tpl[k]];
    if (D.kind != 0) return;
    double al[4];
    for (int m = 0; m < nv; ++m) {
        long long v0 = M.elements[k];
        if (M.node_off) v0 = M.node_off[v0];
        double a = M.sf[(long long)(m * nv) * Ne + k] * x[v0];
        for (int i = 1; i < nv; ++i) {
            long long vi = M.elements[(long long)i * Ne + k];
            if (M.node_off) vi = M.node_off[vi];
            a = fma(M.sf[(long long)(m * nv + i) * Ne + k], x[vi], a);
        }
        al[m] = a;
    }
    const double s = P.cell_scale ? P.cell_scale[k] : 1.0;
    const double cx = M.cent[k], cy = M.cent[Ne + k];
    const int mn = D.mn;
    const int* bl = S.bnl + D.bnl;
    const double* vec = S.vec + 2 * D.node;
    const long long off = S.cell_off[k];
    for (int q = lane; q < D.nbn; q += 32) {
        const int l = bl[q];
        double px = cx, py = cy;
        if (M.model_type != 1) {
            px = fma(s, vec[l], cx);
            py = fma(s, vec[mn + l], cy);
        }
        x[off + l] = interp_at(nv, al, px, py);
    }
}

void launch_calibrate(const Problem& P, double* x, cudaStream_t s)
{
    count();
    const long long threads = 32LL * P.M.Ne;
    k_calibrate<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(P, x);
}

__global__ void k_water_cells(Problem P, const double* __restrict__ u, double* __restrict__ terms)
{
    const MacroDev& M = P.M;
    const MicroSet& S = P.m;
    const int lane = threadIdx.x & 31;
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (k >= M.Ne) return;
    const int nv = M.nv, Ne = M.Ne;
    const bool learned = S.tpl[S.cell_tpl[k]].kind == 1;
    const TplDesc D = S.tpl[learned ? S.cell_tpl_full[k] : S.cell_tpl[k]];
    const int mn = D.mn;
    const int* bnode = S.bnode + D.node;
    const double* cvm = S.cv + D.node;
    const double* vec = S.vec + 2 * D.node;
    const VGPar& pB = S.cell_par ? S.cell_par[k] : P.pB;
    double al[4];
    for (int m = 0; m < nv; ++m) {
        long long v0 = M.elements[k];
        if (M.node_off) v0 = M.node_off[v0];
        double a = M.sf[(long long)(m * nv) * Ne + k] * u[v0];
        for (int i = 1; i < nv; ++i) {
            long long vi = M.elements[(long long)i * Ne + k];
            if (M.node_off) vi = M.node_off[vi];
            a = fma(M.sf[(long long)(m * nv + i) * Ne + k], u[vi], a);
        }
        al[m] = a;
    }
    const double s = P.cell_scale ? P.cell_scale[k] : 1.0;
    const double cx = M.cent[k], cy = M.cent[Ne + k];
    const long long off = S.cell_off[k];
    double p = 0.0;
    for (int l = lane; l < mn; l += 32) {
        double hl;
        if (bnode[l]) {
            double px = cx, py = cy;
            if (M.model_type != 1) {
                px = fma(s, vec[l], cx);
                py = fma(s, vec[mn + l], cy);
            }
            hl = interp_at(nv, al, px, py);
        } else if (learned) {
            p = p + u[off] * cvm[l];
            continue;
        } else {
            hl = u[off + l];
        }
        double Se = vg_se(hl, pB, &d_tables);
        p = p + fma(pB.dth, Se, pB.thr) * cvm[l];
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) p = p + __shfl_xor_sync(0xffffffffu, p, d);
    if (lane == 0) {
        double area = M.scv[k];
        for (int j = 1; j < nv; ++j) area += M.scv[(long long)j * Ne + k];
        terms[water_slot_cell(M, k)] = (area * M.inv_Y) * ((s * s) * p);
    }
}

// ---- learned closure ---------------------------------------------------------
__device__ __forceinline__ double cell_centre_head(const MacroDev& M, const double* u, int k)
{
    const int nv = M.nv, Ne = M.Ne;
    double al[4];
    for (int m = 0; m < nv; ++m) {
        long long v0 = M.elements[k];
        if (M.node_off) v0 = M.node_off[v0];
        double a = M.sf[(long long)(m * nv) * Ne + k] * u[v0];
        for (int i = 1; i < nv; ++i) {
            long long vi = M.elements[(long long)i * Ne + k];
            if (M.node_off) vi = M.node_off[vi];
            a = fma(M.sf[(long long)(m * nv + i) * Ne + k], u[vi], a);
        }
        al[m] = a;
    }
    return interp_at(nv, al, M.cent[k], M.cent[Ne + k]);
}

// one warp per cell; lane-ordered sums over the interior nodes
__global__ void k_cell_summary(Problem P, const double* __restrict__ u, const double* __restrict__ g,
                               const double* __restrict__ qlog, double* __restrict__ out)
{
    const MacroDev& M = P.M;
    const MicroSet& S = P.m;
    const int lane = threadIdx.x & 31;
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (k >= M.Ne) return;
    const VGPar& pB = S.cell_par ? S.cell_par[k] : P.pB;
    const long long off = S.cell_off[k];
    const TplDesc D = S.tpl[S.cell_tpl[k]];
    double th, rate;
    if (D.kind == 1) {
        th = u[off];
        rate = g ? g[off] : 0.0;
    } else {
        const int mn = D.mn;
        const int* bnode = S.bnode + D.node;
        const double* cvm = S.cv + D.node;
        double pw = 0.0, pt = 0.0, pr = 0.0;
        for (int l = lane; l < mn; l += 32) {
            if (bnode[l]) continue;
            const double h = u[off + l];
            double K, Cn, Cd;
            vg_full(h, pB, &d_tables, K, Cn, Cd);
            const double Se = vg_se(h, pB, &d_tables);
            const double A = cvm[l];
            pw = pw + A;
            pt = pt + fma(pB.dth, Se, pB.thr) * A;
            if (g) pr = pr + ((Cn / Cd) * g[off + l]) * A;
        }
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) {
            pw = pw + __shfl_xor_sync(0xffffffffu, pw, d);
            pt = pt + __shfl_xor_sync(0xffffffffu, pt, d);
            pr = pr + __shfl_xor_sync(0xffffffffu, pr, d);
        }
        th = pt / pw;
        rate = g ? pr / pw : 0.0;
    }
    if (lane == 0) {
        double* o = out + 5LL * k;
        o[0] = cell_centre_head(M, u, k);
        o[1] = th;
        o[2] = rate;
        o[3] = qlog ? qlog[k] : 0.0;
        o[4] = vg_head(th, pB, &d_tables);
    }
}

void launch_cell_summary(const Problem& P, const double* u, const double* g, const double* qlog,
                         double* out, cudaStream_t s)
{
    count();
    k_cell_summary<<<(P.M.Ne * 32 + 127) / 128, 128, 0, s>>>(P, u, g, qlog, out);
}

// Features of a learned cell, standardised: log(-H_c), asinh of the head
// rates over the last 3 accepted steps [m/day], theta, log(-h(theta)).
__device__ void closure_features(const Problem& P, const ClosureDev& C, const double* u, int k, float z[6],
                                 int* ood, double* Hc_out, double* dth_out)
{
    const MicroSet& S = P.m;
    const VGPar& pB = S.cell_par ? S.cell_par[k] : P.pB;
    const double Hc = cell_centre_head(P.M, u, k);
    const double th = u[S.cell_off[k]];
    const double hb = vg_head(th, pB, &d_tables);
    const int nh = C.hcount[k];
    const double* hs = C.hist + 3LL * k;
    const double r1 = nh >= 1 ? (Hc - hs[0]) / (C.t[0] - C.t[1]) : 0.0;
    const double r2 = nh >= 2 ? (hs[0] - hs[1]) / (C.t[1] - C.t[2]) : 0.0;
    const double r3 = nh >= 3 ? (hs[1] - hs[2]) / (C.t[2] - C.t[3]) : 0.0;
    double f[6];
    f[0] = log(fmax(-Hc, 1e-6));
    f[1] = asinh(r1);
    f[2] = asinh(r2);
    f[3] = asinh(r3);
    f[4] = th;
    f[5] = log(fmax(-hb, 1e-6));
    int o = 0;
    for (int i = 0; i < 6; ++i) {
        z[i] = (float)((f[i] - C.fmu[i]) / C.fsd[i]);
        if (!(z[i] >= C.zlo[i] && z[i] <= C.zhi[i])) o = 1;
    }
    *ood = o;
    *Hc_out = Hc;
    *dth_out = fma(pB.dth, vg_se(Hc, pB, &d_tables), pB.thr) - th;
}

// one CTA per 128 learned cells (one thread per cell), the network on
// tcgen05 with its accumulators in tensor memory (tsr_mlp_tc.cuh)
__global__ void __launch_bounds__(128) k_closure_update(Problem P, const double* __restrict__ u, ClosureDev C)
{
    extern __shared__ __align__(1024) unsigned char tcsm[];
    uint32_t* slot = reinterpret_cast<uint32_t*>(tcsm + kTcBar + 8);
    tc_stage_weights(reinterpret_cast<const __nv_bfloat16*>(C.w), tcsm);
    tc_bar_init(tcsm);
    tc_alloc(slot);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *slot;
    const int q = blockIdx.x * kTcRows + threadIdx.x;
    const bool mine = q < C.n;
    const int k = mine ? C.cells[q] : 0;
    float z[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int ood = 0;
    double Hc = 0.0, dth = 0.0;
    if (mine) closure_features(P, C, u, k, z, &ood, &Hc, &dth);
    auto x_at = [&](int, int c) -> float { return z[c]; };
    // network A, then (ensemble) network B on the same tile and tensor memory
    float oa[2] = {0.f, 0.f}, ob[2] = {0.f, 0.f};
    uint32_t phase = 0;
    auto out_a = [&](int, float o1, float o2) {
        oa[0] = o1;
        oa[1] = o2;
    };
    bool ok = tc_forward_tile(tcsm, tmem, C.p, x_at, out_a, phase, C.nflag + 1);
    const bool two = C.w2 != nullptr;
    if (two && ok) {
        tc_stage_weights(reinterpret_cast<const __nv_bfloat16*>(C.w2), tcsm);
        auto out_b = [&](int, float o1, float o2) {
            ob[0] = o1;
            ob[1] = o2;
        };
        ok = tc_forward_tile(tcsm, tmem, C.p2, x_at, out_b, phase, C.nflag + 1);
    }
    if (mine && ok) {
        // the coefficients from the (mean) outputs
        const double ya = (double)oa[0] * C.ysd[0] + C.ymu[0];
        const double y1 = two ? 0.5 * (ya + ((double)ob[0] * C.ysd[0] + C.ymu[0])) : ya;
        const double y2 = two ? 0.5 * (((double)oa[1] * C.ysd[1] + C.ymu[1]) + ((double)ob[1] * C.ysd[1] + C.ymu[1]))
                              : (double)oa[1] * C.ysd[1] + C.ymu[1];
        const double sc = P.cell_scale ? P.cell_scale[k] : 1.0;
        const double kQ = exp(y1);
        // y2 = log of the exchange-to-interior-rate ratio
        const double kT = exp(y1 - y2) / ((sc * sc) * C.aint[P.m.cell_tpl_full[k]]);
        const double d = fabs(dth);
        int flag = ood;
        const double kQold = C.kappa[2 * k];
        // the change of kQ over the last step, once the cell's three-step
        // head history is complete (until then the rate inputs change by
        // construction, not because the closure is failing)
        if (C.hcount[k] >= 3 && kQold > 0.0) {
            const double eta = fabs(kQ - kQold) * d / fmax(kQ * d, C.qfloor);
            if (eta > C.thr) flag = 1;
        }
        // the two networks' inflows apart by more than thr_ens (relative to
        // the inflow or the floor): the prediction is not to be trusted
        if (two) {
            const double qa = exp(ya), qb = exp((double)ob[0] * C.ysd[0] + C.ymu[0]);
            const double eta = fabs(qa - qb) * d / fmax(kQ * d, C.qfloor);
            if (eta > C.thr_ens) flag = 1;
        }
        C.kappa[2 * k] = kQ;
        C.kappa[2 * k + 1] = kT;
        C.hcur[k] = Hc;
        C.flags[k] = flag;
        if (flag) atomicAdd(C.nflag, 1);
    }
    __syncthreads();
    tc_free(tmem);
}

void launch_closure_update(const Problem& P, const double* u, const ClosureDev& C, cudaStream_t s)
{
    if (C.n <= 0) return;
    count();
    k_closure_update<<<(C.n + kTcRows - 1) / kTcRows, kTcRows, kTcSmem, s>>>(P, u, C);
}

__global__ void k_closure_push(ClosureDev C)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= C.n) return;
    const int k = C.cells[q];
    double* h = C.hist + 3LL * k;
    h[2] = h[1];
    h[1] = h[0];
    h[0] = C.hcur[k];
    if (C.hcount[k] < 3) C.hcount[k] += 1;
}

void launch_closure_push(const ClosureDev& C, cudaStream_t s)
{
    if (C.n <= 0) return;
    count();
    k_closure_push<<<(C.n + 127) / 128, 128, 0, s>>>(C);
}

// macro part by a strided loop of block 0..; cells one warp each
__global__ void k_relayout(Problem P, int Mn, int Ne, const long long* __restrict__ off_old,
                           const int* __restrict__ learned_old, const long long* __restrict__ off_new,
                           const int* __restrict__ learned_new, const double* __restrict__ summary,
                           const double* __restrict__ u_old, double* __restrict__ u_new)
{
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int nthr = gridDim.x * blockDim.x;
    for (int i = gt; i < Mn; i += nthr) u_new[i] = u_old[i];
    const int lane = threadIdx.x & 31;
    const int k = gt >> 5;
    if (k >= Ne) return;
    const MicroSet& S = P.m;
    const int mn = S.tpl[S.cell_tpl_full[k]].mn;
    const long long a = off_old[k], b = off_new[k];
    const int lo = learned_old[k], ln = learned_new[k];
    if (lo == ln) {
        const int n = lo ? 1 : mn;
        for (int l = lane; l < n; l += 32) u_new[b + l] = u_old[a + l];
    } else if (ln) {
        if (lane == 0) u_new[b] = summary[5LL * k + 1];
    } else {
        const VGPar& pB = S.cell_par ? S.cell_par[k] : P.pB;
        const double hb = vg_head(u_old[a], pB, &d_tables);
        for (int l = lane; l < mn; l += 32) u_new[b + l] = hb;
    }
}

void launch_relayout(const Problem& P, int Mn, int Ne, const long long* off_old, const int* learned_old,
                     const long long* off_new, const int* learned_new, const double* summary,
                     const double* u_old, double* u_new, cudaStream_t s)
{
    count();
    k_relayout<<<(Ne * 32 + 127) / 128, 128, 0, s>>>(P, Mn, Ne, off_old, learned_old, off_new, learned_new,
                                                      summary, u_old, u_new);
}

void launch_water_terms(const Problem& P, const double* u, double* terms, cudaStream_t s)
{
    count(2);
    k_water_macro<<<(P.M.Mn + 127) / 128, 128, 0, s>>>(P, u, terms);
    k_water_cells<<<(P.M.Ne * 32 + 127) / 128, 128, 0, s>>>(P, u, terms);
}

}  // namespace tsr

namespace tsr {

// FP64 pipe peak: independent DFMA chains, 8 per thread (the bound of the
// right-hand side on GB300).  Returns FP64 instructions per second.
__global__ void k_fp64_peak(double* out, double a, double b, int iters)
{
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1.0, x2 = x0 + 2.0, x3 = x0 + 3.0;
    double x4 = x0 + 4.0, x5 = x0 + 5.0, x6 = x0 + 6.0, x7 = x0 + 7.0;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 1234.5678) out[0] = s;
}

int measure_fp64_peak(double* ops_per_s)
{
    int nsm = 0, dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
    double* d = nullptr;
    if (cudaMalloc(&d, 64) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = nsm * 8, threads = 256, iters = 4096;
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
        cudaEventRecord(e0);
        k_fp64_peak<<<blocks, threads>>>(d, 0.999, 1e-3, iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (cudaGetLastError() != cudaSuccess) return 1;
    *ops_per_s = (double)blocks * threads * iters * 8.0 / (best * 1e-3);
    return 0;
}

}  // namespace tsr
