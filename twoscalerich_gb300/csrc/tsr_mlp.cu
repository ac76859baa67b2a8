// tsr_mlp.cu -- training and inference of the learned closure's network on
// the tensor cores (BF16 operands, FP32 accumulation; tsr_mlp.h).
//
// Training runs layer by layer on batches of B rows held in HBM:
//   forward   Z_l = A_{l-1} W_l^T + b_l, A_l = SiLU(Z_l)   (one warp: 16 rows)
//   loss      mean squared error over the 2 outputs
//   backward  dZ_l = dA_l * SiLU'(Z_l), dA_{l-1} = dZ_l W_l (transposed
//             weight copy), dW_l = dZ_l^T A_{l-1} and db_l = column sums,
//             formed per chunk of 256 rows and summed over the chunks in
//             ascending order (no atomics: training is reproducible)
//   AdamW     on the FP32 master parameters, then the BF16 copies.
// Every GEMM operand is rounded to BF16 where it is loaded, at the same
// points as the fused inference kernel, so the training forward pass and
// inference give the same outputs.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/tsr_capi.h"
#include "tsr_device.h"
#include "tsr_internal.h"
#include "tsr_mlp.h"
#include "tsr_mlp_tc.cuh"

using namespace tsr;

namespace {

constexpr int kRowStride = 8;      // training inputs: 8 floats per row (6 used)
constexpr int kChunk = 256;        // rows per block of the weight-gradient reduction

#define CKM(call)                                                              \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) {                                               \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));     \
            return TSR_ERR_CUDA;                                               \
        }                                                                      \
    } while (0)

// A fragment of rows r0 + g, r0 + g + 8 and columns c0 + 2t.. from a
// row-major FP32 matrix (rows >= nrows and columns >= ncols read as 0)
__device__ __forceinline__ void load_a_rows(const float* X, int ld, int r0, int nrows, int c0, int ncols,
                                            uint32_t a[4])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    auto at = [&](int r, int c) -> float {
        return (r < nrows && c < ncols) ? X[(long long)r * ld + c] : 0.0f;
    };
    const int ra = r0 + g, rb = r0 + g + 8, ca = c0 + 2 * t, cb = c0 + 2 * t + 8;
    a[0] = pack_bf16(at(ra, ca), at(ra, ca + 1));
    a[1] = pack_bf16(at(rb, ca), at(rb, ca + 1));
    a[2] = pack_bf16(at(ra, cb), at(ra, cb + 1));
    a[3] = pack_bf16(at(rb, cb), at(rb, cb + 1));
}

// Y[rows x nout] = X[rows x nin] W^T + b (W bf16 [nout][nin]); with
// SILU also S = SiLU(Y).  One warp per 16 rows.
template <int KB, int NT, bool SILU>
__global__ void k_layer_fwd(const float* __restrict__ X, int ldx, int nin_valid, int rows,
                            const __nv_bfloat16* __restrict__ W, const float* __restrict__ bias,
                            float* __restrict__ Y, float* __restrict__ S)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int r0 = warp * 16;
    if (r0 >= rows) return;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t a[4][4];
#pragma unroll
    for (int k = 0; k < KB; ++k) load_a_rows(X, ldx, r0, rows, 16 * k, nin_valid, a[k]);
    float acc[8][4];
    mlp_layer<KB, NT>(a, W, 16 * KB, bias, acc);
    constexpr int nout = 8 * NT;
#pragma unroll
    for (int n = 0; n < NT; ++n) {
        const int c = 8 * n + 2 * t;
        const int ra = r0 + g, rb = r0 + g + 8;
        if (ra < rows) {
            Y[(long long)ra * nout + c] = acc[n][0];
            Y[(long long)ra * nout + c + 1] = acc[n][1];
            if (SILU) {
                S[(long long)ra * nout + c] = silu_f(acc[n][0]);
                S[(long long)ra * nout + c + 1] = silu_f(acc[n][1]);
            }
        }
        if (rb < rows) {
            Y[(long long)rb * nout + c] = acc[n][2];
            Y[(long long)rb * nout + c + 1] = acc[n][3];
            if (SILU) {
                S[(long long)rb * nout + c] = silu_f(acc[n][2]);
                S[(long long)rb * nout + c + 1] = silu_f(acc[n][3]);
            }
        }
    }
}

// dX[rows x nin] = dZ[rows x nout] W (through WT [nin][nout] bf16); KB
// k-blocks of 16 over nout (nout = 8 pads the second half with zeros), NT
// n-tiles over nin.  No bias.
template <int KB, int NT>
__global__ void k_layer_bwd_data(const float* __restrict__ dZ, int nout, int rows,
                                 const __nv_bfloat16* __restrict__ WT, float* __restrict__ dX)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int r0 = warp * 16;
    if (r0 >= rows) return;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    constexpr int nin = 8 * NT;
    uint32_t a[4][4];
#pragma unroll
    for (int k = 0; k < KB; ++k) load_a_rows(dZ, nout, r0, rows, 16 * k, nout, a[k]);
    float acc[8][4];
#pragma unroll
    for (int n = 0; n < NT; ++n) {
        acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.0f;
#pragma unroll
        for (int k = 0; k < KB; ++k) {
            const __nv_bfloat16* wr = WT + (8 * n + g) * nout + 16 * k;
            uint32_t bf[2];
            bf[0] = *reinterpret_cast<const uint32_t*>(wr + 2 * t);
            bf[1] = (16 * k + 8 < nout) ? *reinterpret_cast<const uint32_t*>(wr + 2 * t + 8) : 0u;
            mma_bf16(acc[n], a[k], bf);
        }
    }
#pragma unroll
    for (int n = 0; n < NT; ++n) {
        const int c = 8 * n + 2 * t;
        const int ra = r0 + g, rb = r0 + g + 8;
        if (ra < rows) {
            dX[(long long)ra * nin + c] = acc[n][0];
            dX[(long long)ra * nin + c + 1] = acc[n][1];
        }
        if (rb < rows) {
            dX[(long long)rb * nin + c] = acc[n][2];
            dX[(long long)rb * nin + c + 1] = acc[n][3];
        }
    }
}

// The chunk's part of dW[nout x nin] = dZ^T X over kChunk rows per block,
// written to dWp + blockIdx.x * kMlpParams (every element of the layer, one
// thread each); k_chunk_sum then adds the chunks in ascending order, so the
// gradient -- and training -- does not depend on the order blocks finish.
// One warp per 16 output rows (m-tile), NT n-tiles over nin.  X row stride ldx.
template <int NT>
__global__ void k_layer_bwd_weight(const float* __restrict__ dZ, int nout, const float* __restrict__ X,
                                   int ldx, int nin_valid, int rows, float* __restrict__ dWp)
{
    float* dW = dWp + (size_t)blockIdx.x * kMlpParams;
    const int mt = threadIdx.x >> 5;                 // m-tile of this warp
    if (16 * mt >= nout) return;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    constexpr int nin = 8 * NT;
    const int i0 = blockIdx.x * kChunk;
    float acc[8][4];
#pragma unroll
    for (int n = 0; n < NT; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.0f;
    auto dz = [&](int i, int o) -> float {
        return (i < rows && o < nout) ? dZ[(long long)i * nout + o] : 0.0f;
    };
    auto xx = [&](int i, int c) -> float {
        return (i < rows && c < nin_valid) ? X[(long long)i * ldx + c] : 0.0f;
    };
    for (int kb = 0; kb < kChunk / 16; ++kb) {
        const int ib = i0 + 16 * kb;
        // A[m = out][k = row] = dZ[row][out]
        uint32_t a[4];
        const int oa = 16 * mt + g, ob = 16 * mt + g + 8;
        const int ka = ib + 2 * t, kc = ib + 2 * t + 8;
        a[0] = pack_bf16(dz(ka, oa), dz(ka + 1, oa));
        a[1] = pack_bf16(dz(ka, ob), dz(ka + 1, ob));
        a[2] = pack_bf16(dz(kc, oa), dz(kc + 1, oa));
        a[3] = pack_bf16(dz(kc, ob), dz(kc + 1, ob));
#pragma unroll
        for (int n = 0; n < NT; ++n) {
            // B[k = row][col = in] = X[row][in]
            uint32_t bf[2];
            const int c = 8 * n + g;
            bf[0] = pack_bf16(xx(ka, c), xx(ka + 1, c));
            bf[1] = pack_bf16(xx(kc, c), xx(kc + 1, c));
            mma_bf16(acc[n], a, bf);
        }
    }
#pragma unroll
    for (int n = 0; n < NT; ++n) {
        const int c = 8 * n + 2 * t;
        const int oa = 16 * mt + g, ob = 16 * mt + g + 8;
        if (oa < nout) {
            dW[oa * nin + c] = acc[n][0];
            dW[oa * nin + c + 1] = acc[n][1];
        }
        if (ob < nout) {
            dW[ob * nin + c] = acc[n][2];
            dW[ob * nin + c + 1] = acc[n][3];
        }
    }
}

// the chunk's part of db[o] = sum over its rows of dZ[row][o], at
// dbp + blockIdx.x * kMlpParams
__global__ void k_bias_grad(const float* __restrict__ dZ, int nout, int rows, float* __restrict__ dbp)
{
    const int o = threadIdx.x;
    if (o >= nout) return;
    const int i0 = blockIdx.x * kChunk;
    const int i1 = min(rows, i0 + kChunk);
    float s = 0.0f;
    for (int i = i0; i < i1; ++i) s += dZ[(long long)i * nout + o];
    dbp[(size_t)blockIdx.x * kMlpParams + o] = s;
}

// g[e] = sum over chunks c = 0, 1, ... of part[c][e] (fixed order)
__global__ void k_chunk_sum(const float* __restrict__ part, int chunks, float* __restrict__ g)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kMlpParams) return;
    float s = 0.0f;
    for (int c = 0; c < chunks; ++c) s += part[(size_t)c * kMlpParams + e];
    g[e] = s;
}

// dZ = dA * SiLU'(Z), SiLU'(z) = s (1 + z (1 - s)), s = 1 / (1 + e^-z)
__global__ void k_silu_bwd(const float* __restrict__ dA, const float* __restrict__ Z, float* __restrict__ dZ,
                           long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float z = Z[i];
        const float s = 1.0f / (1.0f + __expf(-z));
        dZ[i] = dA[i] * (s * (1.0f + z * (1.0f - s)));
    }
}

// squared-error loss of the 2 outputs and its gradient (mean over rows and
// outputs); padding columns get zero gradient
__global__ void k_loss(const float* __restrict__ out, const float* __restrict__ y, int rows,
                       float* __restrict__ dout, float* __restrict__ loss)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    const float scale = 1.0f / (float)(rows * kMlpOut);
    float l = 0.0f;
    for (int j = 0; j < kMlpOutPad; ++j) {
        float d = 0.0f;
        if (j < kMlpOut) {
            d = out[(long long)i * kMlpOutPad + j] - y[(long long)i * kMlpOut + j];
            l += d * d;
        }
        dout[(long long)i * kMlpOutPad + j] = 2.0f * d * scale;
    }
    atomicAdd(loss, l * scale);
}

// rows of the dataset in permuted order
__global__ void k_gather(const float* __restrict__ x, const float* __restrict__ y, const int* __restrict__ idx,
                         int rows, float* __restrict__ bx, float* __restrict__ by)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    const long long r = idx[i];
    for (int j = 0; j < kRowStride; ++j) bx[(long long)i * kRowStride + j] = x[r * kRowStride + j];
    for (int j = 0; j < kMlpOut; ++j) by[(long long)i * kMlpOut + j] = y[r * kMlpOut + j];
}

// AdamW on the FP32 master copy (decoupled weight decay on weights only)
__global__ void k_adamw(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                        float* __restrict__ v, const unsigned char* __restrict__ decay, int n, float lr,
                        float b1, float b2, float eps, float wd, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float upd = (mi * c1) / (sqrtf(vi * c2) + eps);
    if (decay[i]) upd += wd * p[i];
    p[i] -= lr * upd;
}

// BF16 copies: w in parameter-block indexing, wt transposed per layer
__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    w[i] = __float2bfloat16_rn(p[i]);
    const int wo[5] = {kW1, kW2, kW3, kW4, kW5};
    const int bo[5] = {kB1, kB2, kB3, kB4, kB5};
    const int ni[5] = {kMlpInPad, kMlpHidden, kMlpHidden, kMlpHidden, kMlpHidden};
    for (int l = 0; l < 5; ++l)
        if (i >= wo[l] && i < bo[l]) {
            const int q = i - wo[l], o = q / ni[l], c = q - o * ni[l];
            const int no = (bo[l] - wo[l]) / ni[l];
            wt[wo[l] + c * no + o] = w[i];
        }
}

// fused inference: one warp per 16 rows, weights staged in shared memory
__global__ void __launch_bounds__(128) k_mlp_infer(const float* __restrict__ x, int rows,
                                                   const __nv_bfloat16* __restrict__ w,
                                                   const float* __restrict__ p, float* __restrict__ y)
{
    __shared__ __align__(16) __nv_bfloat16 sw[kMlpParams];
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) sw[i] = w[i];
    __syncthreads();
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int r0 = warp * 16;
    if (r0 >= rows) return;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    auto at = [&](int r, int c) -> float {
        return (r < rows && c < kMlpIn) ? x[(long long)r * kRowStride + c] : 0.0f;
    };
    float o[4];
    mlp_forward_warp(at(r0 + g, 2 * t), at(r0 + g, 2 * t + 1), at(r0 + g + 8, 2 * t),
                     at(r0 + g + 8, 2 * t + 1), sw, p, o);
    if (t == 0) {
        if (r0 + g < rows) {
            y[(long long)(r0 + g) * kMlpOut] = o[0];
            y[(long long)(r0 + g) * kMlpOut + 1] = o[1];
        }
        if (r0 + g + 8 < rows) {
            y[(long long)(r0 + g + 8) * kMlpOut] = o[2];
            y[(long long)(r0 + g + 8) * kMlpOut + 1] = o[3];
        }
    }
}

// fused inference on tcgen05 (tsr_mlp_tc.cuh): one CTA per 128 rows
__global__ void __launch_bounds__(128) k_mlp_infer_tc(const float* __restrict__ x, int rows,
                                                      const __nv_bfloat16* __restrict__ w,
                                                      const float* __restrict__ p, float* __restrict__ y,
                                                      int* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + kTcBar + 8);
    tc_stage_weights(w, sm);
    tc_bar_init(sm);
    tc_alloc(slot);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *slot;
    uint32_t phase = 0;
    const int r0 = blockIdx.x * kTcRows;
    auto x_at = [&](int r, int c) -> float {
        return (r0 + r < rows) ? x[(long long)(r0 + r) * kRowStride + c] : 0.0f;
    };
    auto out = [&](int r, float a, float b) {
        if (r0 + r < rows) {
            y[(long long)(r0 + r) * kMlpOut] = a;
            y[(long long)(r0 + r) * kMlpOut + 1] = b;
        }
    };
    tc_forward_tile(sm, tmem, p, x_at, out, phase, err);
    __syncthreads();
    tc_free(tmem);
}

// Failure-path probe of the MMA barrier wait: an mbarrier nothing arrives
// on, polled `limit` times like the network's waits; *err = 1 on expiry.
__global__ void k_mbar_probe(long long limit, int* err)
{
    __shared__ __align__(8) unsigned long long bar;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&bar)), "r"(1u) : "memory");
        long long spins = 0;
        while (!bar_try_wait(smem_u32(&bar), 0u)) {
            if (++spins > limit) {
                *err = 1;
                break;
            }
        }
    }
}

}  // namespace

struct tsr_mlp {
    float *d_p = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;
    unsigned char* d_decay = nullptr;
    __nv_bfloat16 *d_w = nullptr, *d_wt = nullptr;
    float *d_x = nullptr, *d_y = nullptr;     // dataset
    long long n_data = 0;
    int* d_idx = nullptr;
    // batch workspace
    int cap = 0;
    float *b_x = nullptr, *b_y = nullptr, *d_loss = nullptr;
    float *z[5] = {}, *a[5] = {}, *dz = nullptr, *da = nullptr, *dx = nullptr;
    float* gpart = nullptr;      // per-chunk gradient parts [chunks][kMlpParams]
    int step = 0;
    cudaStream_t s = nullptr;
    int* d_err = nullptr;
    // set when a bounded wait of the tcgen05 inference expired (its tensor
    // memory may have been released under MMAs in flight): the network
    // refuses further work
    bool unusable = false;
};

namespace {

void mlp_free_batch(tsr_mlp* m)
{
    float** ps[] = {&m->b_x, &m->b_y, &m->d_loss, &m->dz, &m->da, &m->dx, &m->gpart};
    for (float** p : ps) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    for (int l = 0; l < 5; ++l) {
        if (m->z[l]) cudaFree(m->z[l]);
        if (m->a[l]) cudaFree(m->a[l]);
        m->z[l] = m->a[l] = nullptr;
    }
    m->cap = 0;
}

int mlp_reserve(tsr_mlp* m, int rows)
{
    if (rows <= m->cap) return TSR_OK;
    mlp_free_batch(m);
    const size_t r = (size_t)rows;
    CKM(cudaMalloc(&m->b_x, sizeof(float) * r * kRowStride));
    CKM(cudaMalloc(&m->b_y, sizeof(float) * r * kMlpOut));
    CKM(cudaMalloc(&m->d_loss, sizeof(float) * 4));
    CKM(cudaMalloc(&m->dz, sizeof(float) * r * kMlpHidden));
    CKM(cudaMalloc(&m->da, sizeof(float) * r * kMlpHidden));
    CKM(cudaMalloc(&m->dx, sizeof(float) * r * kMlpHidden));
    CKM(cudaMalloc(&m->gpart, sizeof(float) * ((r + kChunk - 1) / kChunk) * kMlpParams));
    for (int l = 0; l < 5; ++l) {
        const int w = (l == 4) ? kMlpOutPad : kMlpHidden;
        CKM(cudaMalloc(&m->z[l], sizeof(float) * r * w));
        CKM(cudaMalloc(&m->a[l], sizeof(float) * r * w));
    }
    m->cap = rows;
    return TSR_OK;
}

int warps_grid(int rows) { return (rows + 63) / 64; }   // 128 threads = 4 warps of 16 rows

// forward of a batch already in b_x; z[l] pre-activations, a[l] = SiLU(z[l])
void forward_batch(tsr_mlp* m, int rows)
{
    const int gb = warps_grid(rows);
    k_layer_fwd<1, 8, true><<<gb, 128, 0, m->s>>>(m->b_x, kRowStride, kMlpIn, rows, m->d_w + kW1,
                                                 m->d_p + kB1, m->z[0], m->a[0]);
    k_layer_fwd<4, 8, true><<<gb, 128, 0, m->s>>>(m->a[0], kMlpHidden, kMlpHidden, rows, m->d_w + kW2,
                                                 m->d_p + kB2, m->z[1], m->a[1]);
    k_layer_fwd<4, 8, true><<<gb, 128, 0, m->s>>>(m->a[1], kMlpHidden, kMlpHidden, rows, m->d_w + kW3,
                                                 m->d_p + kB3, m->z[2], m->a[2]);
    k_layer_fwd<4, 8, true><<<gb, 128, 0, m->s>>>(m->a[2], kMlpHidden, kMlpHidden, rows, m->d_w + kW4,
                                                 m->d_p + kB4, m->z[3], m->a[3]);
    k_layer_fwd<4, 1, false><<<gb, 128, 0, m->s>>>(m->a[3], kMlpHidden, kMlpHidden, rows, m->d_w + kW5,
                                                  m->d_p + kB5, m->z[4], nullptr);
}

// loss and gradients of a batch in b_x / b_y into d_g (zeroed first)
int grad_batch(tsr_mlp* m, int rows)
{
    const int chunks = (rows + kChunk - 1) / kChunk;
    CKM(cudaMemsetAsync(m->gpart, 0, sizeof(float) * (size_t)chunks * kMlpParams, m->s));
    CKM(cudaMemsetAsync(m->d_loss, 0, sizeof(float), m->s));
    forward_batch(m, rows);
    const int gb = warps_grid(rows);
    k_loss<<<(rows + 255) / 256, 256, 0, m->s>>>(m->z[4], m->b_y, rows, m->dz, m->d_loss);
    // layer 5: dz holds dOut [rows x 8]
    k_layer_bwd_weight<8><<<chunks, 32, 0, m->s>>>(m->dz, kMlpOutPad, m->a[3], kMlpHidden, kMlpHidden, rows,
                                                   m->gpart + kW5);
    k_bias_grad<<<chunks, 64, 0, m->s>>>(m->dz, kMlpOutPad, rows, m->gpart + kB5);
    k_layer_bwd_data<1, 8><<<gb, 128, 0, m->s>>>(m->dz, kMlpOutPad, rows, m->d_wt + kW5, m->da);
    const int wo[4] = {kW1, kW2, kW3, kW4};
    const int bo[4] = {kB1, kB2, kB3, kB4};
    const long long nh = (long long)rows * kMlpHidden;
    for (int l = 3; l >= 0; --l) {
        k_silu_bwd<<<(int)std::min<long long>((nh + 255) / 256, 4096), 256, 0, m->s>>>(m->da, m->z[l], m->dz, nh);
        const float* xin = (l == 0) ? m->b_x : m->a[l - 1];
        if (l == 0)
            k_layer_bwd_weight<2><<<chunks, 128, 0, m->s>>>(m->dz, kMlpHidden, xin, kRowStride, kMlpIn, rows,
                                                            m->gpart + wo[l]);
        else
            k_layer_bwd_weight<8><<<chunks, 128, 0, m->s>>>(m->dz, kMlpHidden, xin, kMlpHidden, kMlpHidden, rows,
                                                            m->gpart + wo[l]);
        k_bias_grad<<<chunks, 64, 0, m->s>>>(m->dz, kMlpHidden, rows, m->gpart + bo[l]);
        if (l > 0) k_layer_bwd_data<4, 8><<<gb, 128, 0, m->s>>>(m->dz, kMlpHidden, rows, m->d_wt + wo[l], m->da);
    }
    k_chunk_sum<<<(kMlpParams + 255) / 256, 256, 0, m->s>>>(m->gpart, chunks, m->d_g);
    CKM(cudaGetLastError());
    return TSR_OK;
}

int refresh_bf16(tsr_mlp* m)
{
    k_to_bf16<<<(kMlpParams + 255) / 256, 256, 0, m->s>>>(m->d_p, m->d_w, m->d_wt);
    CKM(cudaGetLastError());
    return TSR_OK;
}

}  // namespace

extern "C" int tsr_mlp_num_params(void) { return kMlpParams; }

extern "C" tsr_mlp* tsr_mlp_create(void)
{
    tsr_mlp* m = new tsr_mlp();
    bool ok = cudaStreamCreateWithFlags(&m->s, cudaStreamNonBlocking) == cudaSuccess;
    const size_t pb = sizeof(float) * kMlpParams;
    ok = ok && cudaMalloc(&m->d_p, pb) == cudaSuccess && cudaMalloc(&m->d_g, pb) == cudaSuccess &&
         cudaMalloc(&m->d_m, pb) == cudaSuccess && cudaMalloc(&m->d_v, pb) == cudaSuccess &&
         cudaMalloc(&m->d_decay, kMlpParams) == cudaSuccess &&
         cudaMalloc(&m->d_w, sizeof(__nv_bfloat16) * kMlpParams) == cudaSuccess &&
         cudaMalloc(&m->d_wt, sizeof(__nv_bfloat16) * kMlpParams) == cudaSuccess &&
         cudaMalloc(&m->d_err, sizeof(int)) == cudaSuccess && cudaMemset(m->d_err, 0, sizeof(int)) == cudaSuccess;
    if (ok) {
        std::vector<unsigned char> dec(kMlpParams, 0);
        const int wo[5] = {kW1, kW2, kW3, kW4, kW5};
        const int bo[5] = {kB1, kB2, kB3, kB4, kB5};
        for (int l = 0; l < 5; ++l)
            for (int i = wo[l]; i < bo[l]; ++i) dec[i] = 1;
        ok = cudaMemset(m->d_p, 0, pb) == cudaSuccess && cudaMemset(m->d_m, 0, pb) == cudaSuccess &&
             cudaMemset(m->d_v, 0, pb) == cudaSuccess &&
             cudaMemset(m->d_wt, 0, sizeof(__nv_bfloat16) * kMlpParams) == cudaSuccess &&
             cudaMemcpy(m->d_decay, dec.data(), kMlpParams, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (!ok) {
        set_error("tsr_mlp_create: device allocation failed");
        tsr_mlp_free(m);
        return nullptr;
    }
    refresh_bf16(m);
    return m;
}

extern "C" void tsr_mlp_free(tsr_mlp* m)
{
    if (!m) return;
    if (m->s) cudaStreamSynchronize(m->s);
    mlp_free_batch(m);
    void* ps[] = {m->d_p, m->d_g, m->d_m, m->d_v, m->d_decay, m->d_w, m->d_wt, m->d_x, m->d_y, m->d_idx, m->d_err};
    for (void* p : ps)
        if (p) cudaFree(p);
    if (m->s) cudaStreamDestroy(m->s);
    delete m;
}

extern "C" int tsr_mlp_set_params(tsr_mlp* m, const float* host)
{
    if (!m || !host) return TSR_ERR_ARG;
    CKM(cudaMemcpyAsync(m->d_p, host, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, m->s));
    CKM(cudaMemsetAsync(m->d_m, 0, sizeof(float) * kMlpParams, m->s));
    CKM(cudaMemsetAsync(m->d_v, 0, sizeof(float) * kMlpParams, m->s));
    m->step = 0;
    int rc = refresh_bf16(m);
    if (rc) return rc;
    CKM(cudaStreamSynchronize(m->s));
    return TSR_OK;
}

extern "C" int tsr_mlp_get_params(tsr_mlp* m, float* host)
{
    if (!m || !host) return TSR_ERR_ARG;
    CKM(cudaMemcpyAsync(host, m->d_p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, m->s));
    CKM(cudaStreamSynchronize(m->s));
    return TSR_OK;
}

// device copies for the closure kernels (bf16 weights, FP32 biases)
namespace tsr {
const void* mlp_device_weights(const tsr_mlp* m) { return m ? m->d_w : nullptr; }
const float* mlp_device_params(const tsr_mlp* m) { return m ? m->d_p : nullptr; }
cudaStream_t mlp_stream(const tsr_mlp* m) { return m ? m->s : nullptr; }
}  // namespace tsr

extern "C" int tsr_mlp_forward(tsr_mlp* m, const float* x_host, int n, float* y_host, int fused)
{
    if (!m || !x_host || !y_host || n < 0) return TSR_ERR_ARG;
    if (m->unusable) {
        set_error("network unusable after an expired tensor-core wait; free it and create a new one");
        return TSR_ERR_TIMEOUT;
    }
    if (n == 0) return TSR_OK;
    int rc = mlp_reserve(m, n);
    if (rc) return rc;
    CKM(cudaMemcpyAsync(m->b_x, x_host, sizeof(float) * (size_t)n * kRowStride, cudaMemcpyHostToDevice, m->s));
    if (fused == 2) {
        CKM(cudaMemsetAsync(m->d_err, 0, sizeof(int), m->s));
        k_mlp_infer_tc<<<(n + kTcRows - 1) / kTcRows, 128, kTcSmem, m->s>>>(m->b_x, n, m->d_w, m->d_p, m->b_y,
                                                                           m->d_err);
        CKM(cudaGetLastError());
        int herr = 0;
        CKM(cudaMemcpyAsync(&herr, m->d_err, sizeof(int), cudaMemcpyDeviceToHost, m->s));
        CKM(cudaMemcpyAsync(y_host, m->b_y, sizeof(float) * (size_t)n * kMlpOut, cudaMemcpyDeviceToHost, m->s));
        CKM(cudaStreamSynchronize(m->s));
        if (herr) {
            m->unusable = true;
            set_error("tcgen05 inference: a wait on the MMA barrier expired (network now unusable)");
            return TSR_ERR_TIMEOUT;
        }
        return TSR_OK;
    }
    if (fused) {
        k_mlp_infer<<<warps_grid(n), 128, 0, m->s>>>(m->b_x, n, m->d_w, m->d_p, m->b_y);
        CKM(cudaGetLastError());
        CKM(cudaMemcpyAsync(y_host, m->b_y, sizeof(float) * (size_t)n * kMlpOut, cudaMemcpyDeviceToHost, m->s));
    } else {
        forward_batch(m, n);
        CKM(cudaGetLastError());
        CKM(cudaMemcpy2DAsync(y_host, sizeof(float) * kMlpOut, m->z[4], sizeof(float) * kMlpOutPad,
                              sizeof(float) * kMlpOut, (size_t)n, cudaMemcpyDeviceToHost, m->s));
    }
    CKM(cudaStreamSynchronize(m->s));
    return TSR_OK;
}

extern "C" int tsr_mlp_grad(tsr_mlp* m, const float* x_host, const float* y_host, int n, float* loss,
                            float* grad_host)
{
    if (!m || !x_host || !y_host || n <= 0) return TSR_ERR_ARG;
    int rc = mlp_reserve(m, n);
    if (rc) return rc;
    CKM(cudaMemcpyAsync(m->b_x, x_host, sizeof(float) * (size_t)n * kRowStride, cudaMemcpyHostToDevice, m->s));
    CKM(cudaMemcpyAsync(m->b_y, y_host, sizeof(float) * (size_t)n * kMlpOut, cudaMemcpyHostToDevice, m->s));
    if ((rc = grad_batch(m, n))) return rc;
    if (loss) CKM(cudaMemcpyAsync(loss, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, m->s));
    if (grad_host)
        CKM(cudaMemcpyAsync(grad_host, m->d_g, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, m->s));
    CKM(cudaStreamSynchronize(m->s));
    return TSR_OK;
}

extern "C" int tsr_mlp_set_data(tsr_mlp* m, const float* x_host, const float* y_host, long long n)
{
    if (!m || !x_host || !y_host || n <= 0 || n > 0x7fffffffLL) return TSR_ERR_ARG;
    if (m->d_x) cudaFree(m->d_x);
    if (m->d_y) cudaFree(m->d_y);
    if (m->d_idx) cudaFree(m->d_idx);
    m->d_x = m->d_y = nullptr;
    m->d_idx = nullptr;
    CKM(cudaMalloc(&m->d_x, sizeof(float) * (size_t)n * kRowStride));
    CKM(cudaMalloc(&m->d_y, sizeof(float) * (size_t)n * kMlpOut));
    CKM(cudaMalloc(&m->d_idx, sizeof(int) * (size_t)n));
    CKM(cudaMemcpy(m->d_x, x_host, sizeof(float) * (size_t)n * kRowStride, cudaMemcpyHostToDevice));
    CKM(cudaMemcpy(m->d_y, y_host, sizeof(float) * (size_t)n * kMlpOut, cudaMemcpyHostToDevice));
    m->n_data = n;
    return TSR_OK;
}

// One AdamW step with the gradients in d_g.
extern "C" int tsr_mlp_adamw_step(tsr_mlp* m, float lr, float wd)
{
    if (!m) return TSR_ERR_ARG;
    m->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f / (1.0f - std::pow(b1, (float)m->step));
    const float c2 = 1.0f / (1.0f - std::pow(b2, (float)m->step));
    k_adamw<<<(kMlpParams + 255) / 256, 256, 0, m->s>>>(m->d_p, m->d_g, m->d_m, m->d_v, m->d_decay, kMlpParams,
                                                       lr, b1, b2, 1e-8f, wd, c1, c2);
    CKM(cudaGetLastError());
    return refresh_bf16(m);
}

// Minibatch AdamW over the dataset: `epochs` passes in a seeded random
// order, learning rate decayed by a cosine from lr to lr/100.  loss_hist
// (may be NULL) receives the mean batch loss of every epoch.
extern "C" int tsr_mlp_train(tsr_mlp* m, int epochs, int batch, float lr, float wd, unsigned long long seed,
                             float* loss_hist)
{
    if (!m || m->n_data <= 0 || epochs < 1 || batch < 16) return TSR_ERR_ARG;
    const long long n = m->n_data;
    if (batch > n) batch = (int)n;
    int rc = mlp_reserve(m, batch);
    if (rc) return rc;
    const long long nb = n / batch;
    std::vector<int> idx((size_t)n);
    for (long long i = 0; i < n; ++i) idx[(size_t)i] = (int)i;
    std::mt19937_64 rng(seed);
    float* h_loss = nullptr;
    CKM(cudaMallocHost(&h_loss, sizeof(float) * (size_t)nb));
    struct PinnedGuard {
        float* p;
        ~PinnedGuard() { cudaFreeHost(p); }
    } guard{h_loss};
    const long long total = nb * epochs;
    long long it = 0;
    for (int e = 0; e < epochs; ++e) {
        std::shuffle(idx.begin(), idx.end(), rng);
        CKM(cudaMemcpyAsync(m->d_idx, idx.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, m->s));
        CKM(cudaStreamSynchronize(m->s));
        for (long long b = 0; b < nb; ++b, ++it) {
            k_gather<<<(batch + 255) / 256, 256, 0, m->s>>>(m->d_x, m->d_y, m->d_idx + b * batch, batch, m->b_x,
                                                            m->b_y);
            if ((rc = grad_batch(m, batch))) return rc;
            CKM(cudaMemcpyAsync(h_loss + b, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, m->s));
            const double frac = (double)it / (double)std::max<long long>(total - 1, 1);
            const float lr_t = (float)(lr * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(3.14159265358979 * frac))));
            if ((rc = tsr_mlp_adamw_step(m, lr_t, wd))) return rc;
        }
        CKM(cudaStreamSynchronize(m->s));
        double s = 0.0;
        for (long long b = 0; b < nb; ++b) s += h_loss[b];
        if (loss_hist) loss_hist[e] = (float)(s / (double)nb);
    }
    return TSR_OK;
}

// Bounded-wait failure paths, run on purpose: which = 0 the grid barrier of
// the fused Gram-Schmidt kernel (a CTA that never arrives), 1 the tensor-core
// MMA barrier (nothing arrives).  Returns TSR_ERR_TIMEOUT when the wait ran
// out and raised its flag, as it must; the context stays usable.
extern "C" int tsr_wait_probe(int which)
{
    int timed_out = 0;
    if (which == 0) {
        if (tsr::barrier_probe(&timed_out)) {
            set_error("wait probe: CUDA error");
            return TSR_ERR_CUDA;
        }
    } else {
        int* err = nullptr;
        CKM(cudaMalloc(&err, sizeof(int)));
        CKM(cudaMemset(err, 0, sizeof(int)));
        k_mbar_probe<<<1, 32>>>(1LL << 14, err);
        cudaError_t e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(&timed_out, err, sizeof(int), cudaMemcpyDeviceToHost);
        cudaFree(err);
        CKM(e);
    }
    if (timed_out) {
        set_error("wait probe: the bounded wait expired");
        return TSR_ERR_TIMEOUT;
    }
    return TSR_OK;
}
