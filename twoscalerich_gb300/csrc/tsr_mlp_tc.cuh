// tsr_mlp_tc.cuh -- the closure network's inference on the 5th-generation
// tensor cores (tcgen05): one CTA per 128 rows, operands in shared memory,
// accumulators in tensor memory.
//
// Per layer: the 128 x K activation tile A and the N x K weight tile W sit
// in shared memory in the K-major core-matrix layout without swizzle (core
// matrix = 8 rows x 16 bytes stored contiguously; core (i, j), i over rows
// in groups of 8, j over K in groups of 8 elements, at byte (i K/8 + j) 128),
// so a K = 16 step of the MMA reads two cores along K (leading byte offset
// 128) for every group of 8 rows (stride byte offset K/8 x 128).  One
// elected thread issues tcgen05.mma (kind::f16, bf16 x bf16 -> f32,
// M = 128) for every K step and commits to an mbarrier; the four warps then
// read their 32 rows of D from tensor memory (tcgen05.ld 32x32b), add the
// bias, apply SiLU in FP32 and write the BF16 result back as the next
// layer's A tile.  The last layer (2 outputs, padded to N = 16) goes to
// global memory.
//
// Every wait on the mbarrier has an iteration limit; on expiry the kernel
// raises an error flag, stops issuing, frees its tensor memory and returns.
#ifndef TSR_MLP_TC_CUH
#define TSR_MLP_TC_CUH

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "tsr_mlp.h"

namespace tsr {

constexpr int kTcRows = 128;            // rows per CTA (the MMA's M)
constexpr int kTcCols = 64;             // tensor-memory columns allocated
constexpr int kTcOutN = 16;             // last layer's N (2 outputs, zero padded)
constexpr long long kTcSpinLimit = 1LL << 20;   // polls of the MMA barrier (each may suspend briefly)

// shared-memory plan (bytes): weight tiles of the 5 layers, the activation
// tile, the mbarrier and the tensor-memory address
constexpr int kTcW1 = 0;                                   // 64 x 16
constexpr int kTcW2 = kTcW1 + 64 * 16 * 2;                 // 64 x 64
constexpr int kTcW3 = kTcW2 + 64 * 64 * 2;
constexpr int kTcW4 = kTcW3 + 64 * 64 * 2;
constexpr int kTcW5 = kTcW4 + 64 * 64 * 2;                 // 16 x 64
constexpr int kTcA = kTcW5 + kTcOutN * 64 * 2;             // 128 x 64
constexpr int kTcBar = kTcA + kTcRows * 64 * 2;
constexpr int kTcSmem = kTcBar + 16;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, c) of a K-major core-matrix tile with K columns
__device__ __forceinline__ int core_off(int r, int c, int K)
{
    return (((r >> 3) * (K >> 3) + (c >> 3)) << 7) + ((r & 7) << 4) + ((c & 7) << 1);
}

// shared-memory matrix descriptor: start address, leading / stride byte
// offsets (16-byte units), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor of kind::f16: D f32, A and B bf16, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :
        : "r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ bool bar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// 16 columns of this warp's 32 tensor-memory lanes
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float v[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Stage the network's weights (bf16 parameter block w) into the tiles.
__device__ __forceinline__ void tc_stage_weights(const __nv_bfloat16* __restrict__ w, unsigned char* sm)
{
    const int offs[5] = {kTcW1, kTcW2, kTcW3, kTcW4, kTcW5};
    const int wo[5] = {kW1, kW2, kW3, kW4, kW5};
    const int nin[5] = {kMlpInPad, kMlpHidden, kMlpHidden, kMlpHidden, kMlpHidden};
    const int nout[5] = {kMlpHidden, kMlpHidden, kMlpHidden, kMlpHidden, kMlpOutPad};
    const int nrow[5] = {kMlpHidden, kMlpHidden, kMlpHidden, kMlpHidden, kTcOutN};
    for (int l = 0; l < 5; ++l) {
        const int K = nin[l];
        for (int i = threadIdx.x; i < nrow[l] * K; i += blockDim.x) {
            const int r = i / K, c = i - r * K;
            const __nv_bfloat16 v = (r < nout[l]) ? w[wo[l] + r * K + c] : __float2bfloat16_rn(0.0f);
            *reinterpret_cast<__nv_bfloat16*>(sm + offs[l] + core_off(r, c, K)) = v;
        }
    }
}

// Forward pass of the 128 rows of this CTA.  x_at(r, c) gives input c of
// row r (0 beyond the data); out(r, o0, o1) receives the two outputs of
// each row.  Returns false if a wait expired (error already flagged).
template <class XAt, class Out>
__device__ bool tc_forward_tile(unsigned char* sm, uint32_t tmem, const float* __restrict__ p, XAt x_at,
                                Out out, uint32_t& phase, int* err)
{
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row = warp * 32 + lane;
    unsigned char* A = sm + kTcA;
    const uint32_t bar = smem_u32(sm + kTcBar);
    // layer-1 A tile: 16 input columns (6 used)
    for (int c = 0; c < kMlpInPad; ++c)
        *reinterpret_cast<__nv_bfloat16*>(A + core_off(row, c, kMlpInPad)) =
            __float2bfloat16_rn(c < kMlpIn ? x_at(row, c) : 0.0f);
    const int woff[5] = {kTcW1, kTcW2, kTcW3, kTcW4, kTcW5};
    const int bo[5] = {kB1, kB2, kB3, kB4, kB5};
    bool ok = true;
    for (int l = 0; l < 5; ++l) {
        const int K = (l == 0) ? kMlpInPad : kMlpHidden;
        const int N = (l == 4) ? kTcOutN : kMlpHidden;
        // make the generic-proxy writes of A visible to the tensor cores
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (tid == 0) {
            const uint32_t a0 = smem_u32(A), b0 = smem_u32(sm + woff[l]);
            const uint32_t sbo = (uint32_t)(K >> 3) * 128u;
            const uint32_t id = idesc_bf16(kTcRows, N);
            for (int k = 0; k < K / 16; ++k)
                tc_mma(tmem, smem_desc(a0 + 256u * k, 128u, sbo), smem_desc(b0 + 256u * k, 128u, sbo), id,
                       k > 0 ? 1u : 0u);
            tc_commit(bar);
        }
        // wait for the MMAs (bounded)
        long long spins = 0;
        while (!bar_try_wait(bar, phase)) {
            if (++spins > kTcSpinLimit) {
                atomicOr(err, 1);
                ok = false;
                break;
            }
        }
        phase ^= 1u;
        if (!__syncthreads_and(ok ? 1 : 0)) {
            // The wait expired: the committed MMAs may still be writing the
            // accumulators.  Give them one more bounded wait before the
            // caller releases the tensor memory.
            spins = 0;
            while (!bar_try_wait(bar, phase ^ 1u) && ++spins <= kTcSpinLimit) {
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncthreads();
            return false;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        // epilogue: this warp's 32 rows of D
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        if (l < 4) {
            for (int c0 = 0; c0 < N; c0 += 16) {
                float v[16];
                tc_ld16(trow + (uint32_t)c0, v);
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const float z = v[i] + p[bo[l] + c0 + i];
                    *reinterpret_cast<__nv_bfloat16*>(A + core_off(row, c0 + i, kMlpHidden)) =
                        __float2bfloat16_rn(silu_f(z));
                }
            }
        } else {
            float v[16];
            tc_ld16(trow, v);
            out(row, v[0] + p[kB5], v[1] + p[kB5 + 1]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    }
    __syncthreads();
    return true;
}

// Tensor memory of the CTA: allocated by warp 0 (address written to *slot).
__device__ __forceinline__ void tc_alloc(uint32_t* slot)
{
    if ((threadIdx.x >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(slot)),
                     "r"((uint32_t)kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
}

__device__ __forceinline__ void tc_free(uint32_t tmem)
{
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"((uint32_t)kTcCols)
                     : "memory");
}

__device__ __forceinline__ void tc_bar_init(unsigned char* sm)
{
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(sm + kTcBar)), "r"(1u) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
}

}  // namespace tsr

#endif
