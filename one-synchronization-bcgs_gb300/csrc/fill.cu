// Zeroing of device buffers by a kernel on the caller's stream.
//
// The drivers clear small accumulators (column maxima, tile counters, status
// words) at every block step. A cudaMemsetAsync can be served by a copy engine,
// and in a host-buffer run the copy engines are busy moving X up and Q down in
// gigabyte chunks, so a memset on the compute stream could wait behind them. A
// kernel runs on the SMs and keeps the compute stream off the copy engines.
#include <cstdint>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "kernels.h"

namespace bcgs {

std::atomic<long long> g_aux_launch_count{0};

namespace {

// Bytes [0, head) and [head + 16 n16, head + 16 n16 + tail) one at a time; the
// 16-byte-aligned body with 128-bit stores, grid-strided.
__global__ void __launch_bounds__(256) zero_kernel(unsigned char* __restrict__ p, int head, uint64_t n16, int tail) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if (tid < (uint64_t)head) p[tid] = 0;
    uint4* body = reinterpret_cast<uint4*>(p + head);
    for (uint64_t i = tid; i < n16; i += stride) body[i] = make_uint4(0u, 0u, 0u, 0u);
    if (tid < (uint64_t)tail) p[head + 16 * n16 + tid] = 0;
}

}  // namespace

int zero_async(void* p, size_t bytes, cudaStream_t st) {
    if (bytes == 0) return 0;
    if (p == nullptr) return (int)cudaErrorInvalidValue;
    unsigned char* b = static_cast<unsigned char*>(p);
    size_t head = (16 - ((uintptr_t)b & 15)) & 15;
    if (head > bytes) head = bytes;
    const uint64_t n16 = (bytes - head) / 16;
    const int tail = (int)(bytes - head - 16 * n16);
    // At most 8 CTAs of 256 threads per SM; small buffers take one CTA.
    const uint64_t want = (n16 + 255) / 256;
    const uint64_t cap = (uint64_t)kNumSMsDefault * 8;
    const unsigned grid = (unsigned)(want < 1 ? 1 : (want > cap ? cap : want));
    zero_kernel<<<grid, 256, 0, st>>>(b, (int)head, n16, tail);
    ++g_launch_count;
    ++g_aux_launch_count;
    return (int)cudaGetLastError();
}

namespace {
struct SmemAttr { int dev; const void* fn; int bytes; };
std::vector<SmemAttr> g_smem_attrs;
std::mutex g_smem_mu;
}  // namespace

// cudaFuncAttributeMaxDynamicSharedMemorySize is a per-device setting: a
// process-wide "set once" would leave every GPU but the first at the 48 KB
// default. This records what was set for each (device, kernel).
int smem_attr(const void* fn, int bytes) {
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return (int)ce;
    std::lock_guard<std::mutex> lock(g_smem_mu);
    for (SmemAttr& a : g_smem_attrs) {
        if (a.dev != dev || a.fn != fn) continue;
        if (a.bytes >= bytes) return 0;
        ce = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (ce == cudaSuccess) a.bytes = bytes;
        return (int)ce;
    }
    ce = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (ce == cudaSuccess) g_smem_attrs.push_back({dev, fn, bytes});
    return (int)ce;
}

}  // namespace bcgs
