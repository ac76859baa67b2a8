// tsr_mlp.h -- the learned closure's network: 6 inputs -> 4 hidden layers of
// 64 (SiLU) -> 2 outputs, BF16 weights and activations, FP32 accumulation,
// on the tensor cores (mma.sync m16n8k16, bf16 x bf16 -> f32).
//
// Parameter block (FP32 master copy, flat):
//   W1 [64 x 16] (inputs padded 6 -> 16 with zero columns), b1 [64],
//   W2, W3, W4 [64 x 64], b2, b3, b4 [64],
//   W5 [8 x 64] (outputs padded 2 -> 8 with zero rows), b5 [8].
// W is row-major [out][in] (y = W x + b).  The BF16 copies keep the same
// layout, plus a transposed copy [in][out] for the backward pass.
#ifndef TSR_MLP_H
#define TSR_MLP_H

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace tsr {

constexpr int kMlpIn = 6;
constexpr int kMlpInPad = 16;
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 2;
constexpr int kMlpOutPad = 8;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// D = A B + D for one m16n8k16 tile: A 16x16 bf16 (row-major fragment),
// B 16x8 bf16 (column fragment), D 16x8 f32
__device__ __forceinline__ void mma_bf16(float d[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float silu_f(float z) { return z / (1.0f + __expf(-z)); }

// Offsets of the parameter block, as compile-time constants.
constexpr int kW1 = 0, kB1 = kW1 + kMlpHidden * kMlpInPad;
constexpr int kW2 = kB1 + kMlpHidden, kB2 = kW2 + kMlpHidden * kMlpHidden;
constexpr int kW3 = kB2 + kMlpHidden, kB3 = kW3 + kMlpHidden * kMlpHidden;
constexpr int kW4 = kB3 + kMlpHidden, kB4 = kW4 + kMlpHidden * kMlpHidden;
constexpr int kW5 = kB4 + kMlpHidden, kB5 = kW5 + kMlpOutPad * kMlpHidden;
constexpr int kMlpParams = kB5 + kMlpOutPad;

// One layer for 16 rows: acc[n] (output columns 8n..8n+7) = bias + A W^T
// with A given as KB k-blocks of 16 inputs.  W is [out][nin] bf16.
template <int KB, int NT>
__device__ __forceinline__ void mlp_layer(const uint32_t (&a)[4][4], const __nv_bfloat16* W, int nin,
                                          const float* bias, float (&acc)[8][4])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int n = 0; n < NT; ++n) {
        const float b0 = bias[8 * n + 2 * t], b1 = bias[8 * n + 2 * t + 1];
        acc[n][0] = b0;
        acc[n][1] = b1;
        acc[n][2] = b0;
        acc[n][3] = b1;
#pragma unroll
        for (int k = 0; k < KB; ++k) {
            // B[kk][col] = W[col][kk]: column g of this n-tile is output 8n+g
            const __nv_bfloat16* wr = W + (8 * n + g) * nin + 16 * k;
            uint32_t bf[2];
            bf[0] = *reinterpret_cast<const uint32_t*>(wr + 2 * t);
            bf[1] = *reinterpret_cast<const uint32_t*>(wr + 2 * t + 8);
            mma_bf16(acc[n], a[k], bf);
        }
    }
}

// SiLU of a 16 x 64 accumulator set, repacked as 4 A fragments
__device__ __forceinline__ void silu_pack(const float (&acc)[8][4], uint32_t (&a)[4][4])
{
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        a[p][0] = pack_bf16(silu_f(acc[2 * p][0]), silu_f(acc[2 * p][1]));
        a[p][1] = pack_bf16(silu_f(acc[2 * p][2]), silu_f(acc[2 * p][3]));
        a[p][2] = pack_bf16(silu_f(acc[2 * p + 1][0]), silu_f(acc[2 * p + 1][1]));
        a[p][3] = pack_bf16(silu_f(acc[2 * p + 1][2]), silu_f(acc[2 * p + 1][3]));
    }
}

// Fused forward pass of the whole network for the 16 rows held by one warp.
// in0/in1: the lane's two input values of row g = lane/4 (features 2t, 2t+1,
// t = lane % 4; zero for t = 3) and in2/in3 the same of row g + 8.  Weights
// w (bf16, parameter-block indexing; shared or global memory) and FP32
// biases p.  Outputs of row g are o[0], o[1] and of row g + 8 o[2], o[3]
// on lanes with t == 0.
//
// Register layout of m16n8k16 (g = lane / 4, t = lane % 4): A holds rows
// g, g+8 at columns 2t, 2t+1 (a0, a1) and 2t+8, 2t+9 (a2, a3); B holds
// rows 2t, 2t+1 (b0) and 2t+8, 2t+9 (b1) of column g; D holds rows g, g+8
// at columns 2t, 2t+1.  The D tiles of output columns [16p, 16p+8) and
// [16p+8, 16p+16) are therefore exactly the A fragment of input columns
// [16p, 16p+16) of the next layer, so activations never leave registers.
__device__ __forceinline__ void mlp_forward_warp(float in0, float in1, float in2, float in3,
                                                 const __nv_bfloat16* w, const float* p, float o[4])
{
    uint32_t a[4][4];
    a[0][0] = pack_bf16(in0, in1);
    a[0][1] = pack_bf16(in2, in3);
    a[0][2] = 0u;
    a[0][3] = 0u;
    float acc[8][4];
    mlp_layer<1, 8>(a, w + kW1, kMlpInPad, p + kB1, acc);
    silu_pack(acc, a);
    mlp_layer<4, 8>(a, w + kW2, kMlpHidden, p + kB2, acc);
    silu_pack(acc, a);
    mlp_layer<4, 8>(a, w + kW3, kMlpHidden, p + kB3, acc);
    silu_pack(acc, a);
    mlp_layer<4, 8>(a, w + kW4, kMlpHidden, p + kB4, acc);
    silu_pack(acc, a);
    mlp_layer<4, 1>(a, w + kW5, kMlpHidden, p + kB5, acc);
    o[0] = acc[0][0];
    o[1] = acc[0][1];
    o[2] = acc[0][2];
    o[3] = acc[0][3];
}

}  // namespace tsr

#endif
