// tsr_noalloc.cu -- the fixed-order FP64 dot product for callers that must
// not allocate device memory.
//
// Who needs it: a program that embeds this solver and owns every byte of
// device memory through its own pool hands the library views into memory it
// already holds, and forbids allocations behind its back; and latency-
// critical loops cannot afford the device-wide synchronisation a
// cudaMalloc/cudaFree pair can cause.  The library's
// usual entry points keep their scratch in buffers that tsr_init allocates;
// this one needs no context and no allocation at all.
//
// How: the block partial sums and the completion counter of the reduction
// live in the file-scope array below, a fixed 64 KB (plus a 256-byte slot
// for the counter) that every GPU loading the library holds until the
// process exits.  Host code cannot use the array's name as a device address,
// so the first call on each device, with that device current, asks the
// runtime for the array's device address (cudaGetSymbolAddress) and keeps
// it.  Make that first call before any stream capture begins.
//
// The result equals tsr_dot's bit for bit: the same chunk, lane and warp
// order (block b sums items 8192 b + 256 s + t, warps combine by xor
// butterfly, the eight warp sums pairwise, the last block reduces the block
// sums the same way).
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/tsr_capi.h"
#include "tsr_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 8192;                       // items per block
constexpr int kMaxBlocks = 8192;                   // block partials the array holds
constexpr long long kMaxN = (long long)kMaxBlocks * kChunk;   // 67,108,864 items
constexpr int kCounterSlot = kMaxBlocks;           // counter lives after the partials
constexpr int kScratchDoubles = kMaxBlocks + 32;   // + one 256-byte slot
constexpr int kMaxDevices = 64;

}  // namespace

// The shared scratch: [0, kMaxBlocks) block partials, then the counter.
static __device__ __align__(256) double tsr_noalloc_scratch[kScratchDoubles];

namespace {

__device__ __forceinline__ double block_sum(double a, double* ws)
{
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) a = a + __shfl_xor_sync(0xffffffffu, a, d);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = a;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) r = ((ws[0] + ws[1]) + (ws[2] + ws[3])) + ((ws[4] + ws[5]) + (ws[6] + ws[7]));
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kThreads) k_dot_noalloc(const double* __restrict__ x,
                                                          const double* __restrict__ y,
                                                          long long n, double* scratch,
                                                          double* out)
{
    __shared__ double ws[8];
    __shared__ int last;
    double* partials = scratch;
    unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + kCounterSlot);
    const long long base = (long long)blockIdx.x * kChunk + threadIdx.x;
    double a = 0.0;
    for (int s = 0; s < kChunk / kThreads; ++s) {
        const long long i = base + (long long)s * kThreads;
        if (i < n) a = fma(x[i], y[i], a);
    }
    double r = block_sum(a, ws);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = r;
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double b = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += kThreads) b = b + __ldcg(partials + i);
    double tot = block_sum(b, ws);
    if (threadIdx.x == 0) {
        *out = tot;
        *counter = 0u;    // ready for the next call
    }
}

std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up
// once per device).
int scratch_for_current_device(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        tsr::set_error(std::string("tsr_dot_device_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return TSR_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        tsr::set_error("tsr_dot_device_noalloc: device index out of range");
        return TSR_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, tsr_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            tsr::set_error(std::string("tsr_dot_device_noalloc: cudaGetSymbolAddress: ") +
                           cudaGetErrorString(e));
            return TSR_ERR_CUDA;
        }
        g_scratch[dev] = static_cast<double*>(p);
    }
    *out = g_scratch[dev];
    return TSR_OK;
}

}  // namespace

extern "C" int tsr_dot_device_noalloc(const double* d_x, const double* d_y, long long n,
                                      double* d_out, void* stream)
{
    if (n < 0 || !d_out || (n > 0 && (!d_x || !d_y))) {
        tsr::set_error("tsr_dot_device_noalloc: invalid arguments");
        return TSR_ERR_ARG;
    }
    if (n > kMaxN) {
        tsr::set_error("tsr_dot_device_noalloc: n = " + std::to_string(n) +
                       " exceeds the maximum of " + std::to_string(kMaxN) +
                       " elements that its fixed scratch array supports");
        return TSR_ERR_ARG;
    }
    double* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != TSR_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (n == 0) {
        e = cudaMemsetAsync(d_out, 0, sizeof(double), s);   // the empty sum is +0.0
    } else {
        // the counter must start at zero
        e = cudaMemsetAsync(scratch + kCounterSlot, 0, sizeof(unsigned int), s);
        if (e == cudaSuccess) {
            const int blocks = (int)((n + kChunk - 1) / kChunk);
            k_dot_noalloc<<<blocks, kThreads, 0, s>>>(d_x, d_y, n, scratch, d_out);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        tsr::set_error(std::string("tsr_dot_device_noalloc: ") + cudaGetErrorString(e));
        return TSR_ERR_CUDA;
    }
    return TSR_OK;
}
