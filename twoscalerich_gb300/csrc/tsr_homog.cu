// tsr_homog.cu -- effective conductivity Keff(h) of the macro continuum by
// homogenisation of the unit cell, the step the reference leaves to a
// MATLAB script it does not ship (src/main.cpp:111-112, "see Keff/run.m").
//
// The macro continuum is the connected material A around the inclusions
// (material B, whose exchange the micro cells carry).  Its effective
// conductivity is K_A(h) times the homogenised tensor of the perforated
// cell: for each direction d, find the Y-periodic chi_d with
//     div (grad chi_d + e_d) = 0 in Y_A,   (grad chi_d + e_d) . n = 0 on the
// inclusion boundaries, and
//     Khom_cd = (1/|Y|) int_{Y_A} (e_c . (grad chi_d + e_d)) dy.
// The reference's own table (tests/Richards_Equation/Keff.txt) has exactly
// this structure: every row is K_A(10^logh) times one constant tensor.
//
// Discretisation (this project's own): cell-centred finite volumes on an
// Mx x My grid over the cell, periodic; the face between two grid cells
// carries the fraction of its length that lies in Y_A (computed exactly by
// clipping the face against the inclusion's triangles), so the inclusion
// boundary enters as a cut-face no-flux condition.  The symmetric
// positive semi-definite system is solved by conjugate gradients with a
// Jacobi preconditioner on the GPU (matrix-free 5-point stencil), every
// reduction in a fixed order (two stages, fixed block size), so the result
// is reproducible bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tsr_capi.h"
#include "tsr_internal.h"
#include "tsr_math.h"

namespace {

constexpr int kHT = 256;            // threads per block of the solver kernels

// y = L x with L phi_P = sum over faces w_f (phi_P - phi_Q); rows of cells
// cut off from the rest (all four weights zero) are the identity
__global__ void k_hmatvec(int Mx, int My, const double* __restrict__ wx, const double* __restrict__ wy,
                          const double* __restrict__ x, double* __restrict__ y)
{
    const long long n = (long long)Mx * My;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int i = (int)(p % Mx), j = (int)(p / Mx);
    const int im = i == 0 ? Mx - 1 : i - 1, ip = i == Mx - 1 ? 0 : i + 1;
    const int jm = j == 0 ? My - 1 : j - 1, jp = j == My - 1 ? 0 : j + 1;
    const long long pe = (long long)j * Mx + ip, pw = (long long)j * Mx + im;
    const long long pn = (long long)jp * Mx + i, ps = (long long)jm * Mx + i;
    const double we = wx[p], ww = wx[pw], wn = wy[p], wsth = wy[ps];
    const double xp = x[p];
    const double d = (we + ww) + (wn + wsth);
    if (d == 0.0) {
        y[p] = xp;
        return;
    }
    double a = we * (xp - x[pe]);
    a = fma(ww, xp - x[pw], a);
    a = fma(wn, xp - x[pn], a);
    a = fma(wsth, xp - x[ps], a);
    y[p] = a;
}

// block partials of sum x_i y_i (or x_i y_i / d_i when d is given): thread
// t of block b sums items b*kHT*8 + q*kHT + t, q ascending; warp xor
// butterfly; warps pairwise
__global__ void k_hdot(long long n, const double* __restrict__ x, const double* __restrict__ y,
                       const double* __restrict__ dinv, double* __restrict__ part)
{
    __shared__ double ws[kHT / 32];
    const long long base = (long long)blockIdx.x * kHT * 8 + threadIdx.x;
    double a = 0.0;
    for (int q = 0; q < 8; ++q) {
        const long long i = base + (long long)q * kHT;
        if (i < n) {
            const double v = dinv ? x[i] * dinv[i] : x[i];
            a = fma(v, y[i], a);
        }
    }
    for (int d = 16; d >= 1; d >>= 1) a = a + __shfl_xor_sync(0xffffffffu, a, d);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = ((ws[0] + ws[1]) + (ws[2] + ws[3])) + ((ws[4] + ws[5]) + (ws[6] + ws[7]));
        part[blockIdx.x] = r;
    }
}

// one block: the sum of nb partials in a fixed order, into *out
__global__ void k_hsum(int nb, const double* __restrict__ part, double* __restrict__ out)
{
    __shared__ double ws[kHT / 32];
    double a = 0.0;
    for (int i = threadIdx.x; i < nb; i += kHT) a = a + part[i];
    for (int d = 16; d >= 1; d >>= 1) a = a + __shfl_xor_sync(0xffffffffu, a, d);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) *out = ((ws[0] + ws[1]) + (ws[2] + ws[3])) + ((ws[4] + ws[5]) + (ws[6] + ws[7]));
}

// x += alpha p; r -= alpha q  (alpha = s[0] / s[1]; 0 once p vanishes)
__global__ void k_hupdate(long long n, const double* __restrict__ s, double* __restrict__ x,
                          const double* __restrict__ p, double* __restrict__ r, const double* __restrict__ q)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double alpha = s[1] != 0.0 ? s[0] / s[1] : 0.0;
    x[i] = fma(alpha, p[i], x[i]);
    r[i] = fma(-alpha, q[i], r[i]);
}

// p = r / d + beta p  (beta = s[2] / s[0]; the caller then sets s[0] <- s[2])
__global__ void k_hdir(long long n, const double* __restrict__ s, const double* __restrict__ r,
                       const double* __restrict__ dinv, double* __restrict__ p)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double beta = s[0] != 0.0 ? s[2] / s[0] : 0.0;
    p[i] = fma(beta, p[i], r[i] * dinv[i]);
}

__global__ void k_hshift(double* s) { s[0] = s[2]; }

// length of the part of segment [a, b] (axis-aligned, coordinate `along`
// varying) inside triangle (x, y); `fixed` is the other coordinate
double clip_len(double fixed, double a, double b, bool xface, const double* tx, const double* ty)
{
    // the triangle's cross-section at the fixed coordinate is an interval
    double lo = 1e300, hi = -1e300;
    int hits = 0;
    for (int e = 0; e < 3; ++e) {
        const int f = (e + 1) % 3;
        // xface: the face is x = fixed, y in [a, b]; else y = fixed, x in [a, b]
        const double c0 = xface ? tx[e] : ty[e], c1 = xface ? tx[f] : ty[f];
        const double o0 = xface ? ty[e] : tx[e], o1 = xface ? ty[f] : tx[f];
        if ((c0 - fixed) * (c1 - fixed) > 0.0) continue;
        if (c0 == c1) {
            if (c0 != fixed) continue;
            lo = std::min(lo, std::min(o0, o1));
            hi = std::max(hi, std::max(o0, o1));
            hits += 2;
            continue;
        }
        const double s = (fixed - c0) / (c1 - c0);
        const double o = o0 + s * (o1 - o0);
        lo = std::min(lo, o);
        hi = std::max(hi, o);
        ++hits;
    }
    if (hits < 2) return 0.0;
    const double l = std::min(hi, b) - std::max(lo, a);
    return l > 0.0 ? l : 0.0;
}

}  // namespace

extern "C" int tsr_keff_homogenize(const micro_mesh_struct* inclusion, double cell_width, double cell_height,
                                   int resolution, double tol, const soil_struct* soilA, double factor,
                                   double logh_first, double logr, int n_h, double* Khom,
                                   double* epsA, double* table)
{
    if (!inclusion || !Khom || !epsA || resolution < 8 || resolution > 8192 || !(cell_width > 0.0) ||
        !(cell_height > 0.0) || inclusion->no_verts != 3 || n_h < 0 || (n_h > 0 && (!soilA || !table))) {
        tsr::set_error("tsr_keff_homogenize: invalid arguments");
        return TSR_ERR_ARG;
    }
    const micro_mesh_struct& m = *inclusion;
    const int Mx = resolution;
    const int My = std::max(8, (int)std::lround(resolution * cell_height / cell_width));
    const double hx = cell_width / Mx, hy = cell_height / My;
    const long long n = (long long)Mx * My;
    const int Ne = m.no_elements, mn = m.no_nodes;
    // area of material A
    double area_b = 0.0;
    for (int e = 0; e < Ne; ++e) {
        const int a = m.elements[e], b = m.elements[Ne + e], c = m.elements[2 * Ne + e];
        const double x0 = m.nodes[a], y0 = m.nodes[mn + a];
        area_b += 0.5 * std::fabs((m.nodes[b] - x0) * (m.nodes[mn + c] - y0) -
                                  (m.nodes[c] - x0) * (m.nodes[mn + b] - y0));
    }
    *epsA = 1.0 - area_b / (cell_width * cell_height);
    // face fractions in A: 1 - (length inside the inclusion's triangles) / face length;
    // triangles bucketed by the grid columns and rows they span
    std::vector<double> fx((size_t)n, 1.0), fy((size_t)n, 1.0);
    std::vector<std::vector<int>> col((size_t)Mx + 1), row((size_t)My + 1);
    for (int e = 0; e < Ne; ++e) {
        double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
        for (int v = 0; v < 3; ++v) {
            const int q = m.elements[(size_t)v * Ne + e];
            xmin = std::min(xmin, m.nodes[q]);
            xmax = std::max(xmax, m.nodes[q]);
            ymin = std::min(ymin, m.nodes[mn + q]);
            ymax = std::max(ymax, m.nodes[mn + q]);
        }
        // x-faces at x = (i+1) hx with xmin <= x <= xmax
        for (int i = std::max(0, (int)std::floor(xmin / hx) - 1); i <= std::min(Mx - 1, (int)std::ceil(xmax / hx)); ++i)
            col[i].push_back(e);
        for (int j = std::max(0, (int)std::floor(ymin / hy) - 1); j <= std::min(My - 1, (int)std::ceil(ymax / hy)); ++j)
            row[j].push_back(e);
    }
    auto tri = [&](int e, double* tx, double* ty) {
        for (int v = 0; v < 3; ++v) {
            const int q = m.elements[(size_t)v * Ne + e];
            tx[v] = m.nodes[q];
            ty[v] = m.nodes[mn + q];
        }
    };
    for (int i = 0; i < Mx; ++i) {
        const double xf = (i + 1) * hx;         // x-face between columns i and i+1 (i = Mx-1: the periodic seam)
        for (int e : col[i]) {
            double tx[3], ty[3];
            tri(e, tx, ty);
            const double ylo = std::min(ty[0], std::min(ty[1], ty[2])), yhi = std::max(ty[0], std::max(ty[1], ty[2]));
            for (int j = std::max(0, (int)std::floor(ylo / hy)); j <= std::min(My - 1, (int)std::floor(yhi / hy)); ++j)
                fx[(size_t)j * Mx + i] -= clip_len(xf, j * hy, (j + 1) * hy, true, tx, ty) / hy;
        }
    }
    for (int j = 0; j < My; ++j) {
        const double yf = (j + 1) * hy;
        for (int e : row[j]) {
            double tx[3], ty[3];
            tri(e, tx, ty);
            const double xlo = std::min(tx[0], std::min(tx[1], tx[2])), xhi = std::max(tx[0], std::max(tx[1], tx[2]));
            for (int i = std::max(0, (int)std::floor(xlo / hx)); i <= std::min(Mx - 1, (int)std::floor(xhi / hx)); ++i)
                fy[(size_t)j * Mx + i] -= clip_len(yf, i * hx, (i + 1) * hx, false, tx, ty) / hx;
        }
    }
    std::vector<double> wx((size_t)n), wy((size_t)n), dinv((size_t)n);
    for (long long p = 0; p < n; ++p) {
        fx[p] = std::min(1.0, std::max(0.0, fx[p]));
        fy[p] = std::min(1.0, std::max(0.0, fy[p]));
        wx[p] = fx[p] * hy / hx;
        wy[p] = fy[p] * hx / hy;
    }
    for (long long p = 0; p < n; ++p) {
        const int i = (int)(p % Mx), j = (int)(p / Mx);
        const long long pw = (long long)j * Mx + (i == 0 ? Mx - 1 : i - 1);
        const long long ps = (long long)(j == 0 ? My - 1 : j - 1) * Mx + i;
        const double d = (wx[p] + wx[pw]) + (wy[p] + wy[ps]);
        dinv[p] = d > 0.0 ? 1.0 / d : 1.0;
    }
    // device buffers
    double *d_wx = nullptr, *d_wy = nullptr, *d_di = nullptr, *d_x = nullptr, *d_r = nullptr, *d_p = nullptr,
           *d_q = nullptr, *d_part = nullptr, *d_s = nullptr;
    const int nblk = (int)((n + kHT - 1) / kHT);
    const int nred = (int)((n + kHT * 8 - 1) / (kHT * 8));
    std::vector<double*> bufs;
    auto alloc = [&](double** p, size_t cnt) {
        cudaError_t e = cudaMalloc(p, sizeof(double) * cnt);
        if (e == cudaSuccess) bufs.push_back(*p);
        return e;
    };
    auto release = [&]() {
        for (double* b : bufs) cudaFree(b);
        bufs.clear();
    };
    cudaError_t ce = cudaSuccess;
    for (auto pr : {std::make_pair(&d_wx, (size_t)n), std::make_pair(&d_wy, (size_t)n),
                    std::make_pair(&d_di, (size_t)n), std::make_pair(&d_x, (size_t)n), std::make_pair(&d_r, (size_t)n),
                    std::make_pair(&d_p, (size_t)n), std::make_pair(&d_q, (size_t)n),
                    std::make_pair(&d_part, (size_t)nred), std::make_pair(&d_s, (size_t)8)})
        if (ce == cudaSuccess) ce = alloc(pr.first, pr.second);
    if (ce == cudaSuccess) ce = cudaMemcpy(d_wx, wx.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(d_wy, wy.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(d_di, dinv.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) {
        release();
        tsr::set_error(std::string("tsr_keff_homogenize: ") + cudaGetErrorString(ce));
        return TSR_ERR_CUDA;
    }
    const long long max_it = 40LL * (Mx + My) + 1000;
    for (int d = 0; d < 2; ++d) {
        // right-hand side: hy (fx_P - fx_W) for d = x, hx (fy_P - fy_S) for d = y
        std::vector<double> rhs((size_t)n);
        double rnorm0 = 0.0;
        for (long long p = 0; p < n; ++p) {
            const int i = (int)(p % Mx), j = (int)(p / Mx);
            const long long pw = (long long)j * Mx + (i == 0 ? Mx - 1 : i - 1);
            const long long ps = (long long)(j == 0 ? My - 1 : j - 1) * Mx + i;
            rhs[p] = d == 0 ? hy * (fx[p] - fx[pw]) : hx * (fy[p] - fy[ps]);
            rnorm0 = std::fma(rhs[p], rhs[p], rnorm0);
        }
        ce = cudaMemcpy(d_r, rhs.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
        if (ce == cudaSuccess) ce = cudaMemset(d_x, 0, sizeof(double) * n);
        if (ce == cudaSuccess) ce = cudaMemset(d_p, 0, sizeof(double) * n);
        if (ce == cudaSuccess) ce = cudaMemset(d_s, 0, sizeof(double) * 8);
        if (ce != cudaSuccess) break;
        // s[0] = r.z (z = D^-1 r), s[1] = p.q, s[2] = the new r.z, s[3] = r.r;
        // start: p = z (beta = 0 while s[0] = 0), s[0] = r.z
        k_hdot<<<nred, kHT>>>(n, d_r, d_r, d_di, d_part);
        k_hsum<<<1, kHT>>>(nred, d_part, d_s + 2);
        k_hdir<<<nblk, kHT>>>(n, d_s, d_r, d_di, d_p);
        k_hshift<<<1, 1>>>(d_s);
        long long it = 0;
        if (!(rnorm0 > 0.0)) it = -1;                       // nothing to solve: chi = 0
        double hs[4] = {0, 0, 0, 0};
        for (; it >= 0 && it < max_it; ++it) {
            k_hmatvec<<<nblk, kHT>>>(Mx, My, d_wx, d_wy, d_p, d_q);
            k_hdot<<<nred, kHT>>>(n, d_p, d_q, nullptr, d_part);
            k_hsum<<<1, kHT>>>(nred, d_part, d_s + 1);
            k_hupdate<<<nblk, kHT>>>(n, d_s, d_x, d_p, d_r, d_q);
            k_hdot<<<nred, kHT>>>(n, d_r, d_r, d_di, d_part);
            k_hsum<<<1, kHT>>>(nred, d_part, d_s + 2);
            k_hdir<<<nblk, kHT>>>(n, d_s, d_r, d_di, d_p);
            k_hshift<<<1, 1>>>(d_s);
            if ((it & 31) == 31) {
                k_hdot<<<nred, kHT>>>(n, d_r, d_r, nullptr, d_part);
                k_hsum<<<1, kHT>>>(nred, d_part, d_s + 3);
                ce = cudaMemcpy(hs, d_s, sizeof(double) * 4, cudaMemcpyDeviceToHost);
                if (ce != cudaSuccess) break;
                if (!(hs[3] > tol * tol * rnorm0)) break;
            }
        }
        if (ce == cudaSuccess) ce = cudaGetLastError();
        if (ce != cudaSuccess) break;
        if (it >= max_it) {          // it = -1: the right-hand side was zero
            release();
            tsr::set_error("tsr_keff_homogenize: conjugate gradients did not converge");
            return TSR_ERR_ARG;
        }
        std::vector<double> x((size_t)n);
        ce = cudaMemcpy(x.data(), d_x, sizeof(double) * n, cudaMemcpyDeviceToHost);
        if (ce != cudaSuccess) break;
        // mean flux (K_A = 1) over the cell: x-faces give component x, y-faces component y
        double qx = 0.0, qy = 0.0;
        for (long long p = 0; p < n; ++p) {
            const int i = (int)(p % Mx), j = (int)(p / Mx);
            const long long pe = (long long)j * Mx + (i == Mx - 1 ? 0 : i + 1);
            const long long pn = (long long)(j == My - 1 ? 0 : j + 1) * Mx + i;
            qx += (wx[p] * (x[pe] - x[p]) + (d == 0 ? fx[p] * hy : 0.0)) * hx;
            qy += (wy[p] * (x[pn] - x[p]) + (d == 1 ? fy[p] * hx : 0.0)) * hy;
        }
        const double area = cell_width * cell_height;
        Khom[0 * 2 + d] = qx / area;   // row x
        Khom[1 * 2 + d] = qy / area;   // row y
    }
    release();
    if (ce != cudaSuccess) {
        tsr::set_error(std::string("tsr_keff_homogenize: ") + cudaGetErrorString(ce));
        return TSR_ERR_CUDA;
    }
    // the table in the reference's layout (component-major, K11 K12 K21 K22):
    // factor * K_A(10^logh) * Khom, K_A the van Genuchten-Mualem conductivity
    if (n_h > 0) {
        static const tsr_math_tables T = TSR_MATH_TABLES_INIT;
        const double nA = soilA->n, mA = soilA->m, al = soilA->alpha, Ks = soilA->Ksat;
        for (int r = 0; r < n_h; ++r) {
            const double logh = logh_first + r * logr;
            const double h = std::pow(10.0, logh);
            const double t = tsr_exp(nA * tsr_log(al * h, &T), &T);
            const double Se = tsr_exp(-mA * tsr_log1p(t, &T), &T);
            const double B = -tsr_expm1(mA * tsr_log(t / (1.0 + t), &T), &T);
            const double KA = Ks * std::sqrt(Se) * B * B;
            table[r] = logh;
            for (int c = 0; c < 4; ++c) table[(size_t)(1 + c) * n_h + r] = factor * KA * Khom[c];
        }
    }
    return TSR_OK;
}
