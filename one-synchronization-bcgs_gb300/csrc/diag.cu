// Diagnostics.
//
// 1. Fill every SM's shared memory with one bit pattern. A kernel that reads
//    shared memory it did not write sees whatever an earlier CTA on that SM left
//    there: harmless leftovers in one run, NaN bit patterns from another stream's
//    kernel in the next. Filling shared memory with NaN before a run makes such
//    reads show up deterministically (tests/test_stale_smem_gpu.py).
// 2. Make one bounded wait run out. One thread waits, with the tensor-core
//    kernels' own bounded wait, on an mbarrier that nothing completes. The wait
//    gives up after its time limit, records its code and returns, and the host
//    reads the code; the context stays usable (tests/test_timeout_gpu.py).
#include "../../include/orth_gb300.h"
#include "common.cuh"
#include "kernels.h"
#include "tc_common.cuh"

namespace bcgs {

__global__ void fill_shared_kernel(unsigned long long bits, int words) {
    extern __shared__ unsigned long long sfill[];
    for (int i = threadIdx.x; i < words; i += blockDim.x) sfill[i] = bits;
    __syncthreads();
}

// out[0]: the error code the bounded wait recorded (-1 if it saw the phase
// complete, which nothing here can cause); out[1]: the abort flag it set.
__global__ void wait_timeout_probe_kernel(int code, int* out) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ volatile int abort_flag;
    __shared__ int err;
    if (threadIdx.x == 0) {
        abort_flag = 0;
        err = 0;
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
        const bool ok = tc::mbar_wait(&bar, 0u, &abort_flag, &err, code);
        out[0] = ok ? -1 : err;
        out[1] = abort_flag;
    }
}

}  // namespace bcgs

extern "C" int orth_gb300_timeout_probe(int code, void* stream, int out[2]) {
    using namespace bcgs;
    if (!out || code == 0) return 2;
    int* d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(int)) != cudaSuccess) return 3;
    cudaStream_t st = (cudaStream_t)stream;
    wait_timeout_probe_kernel<<<1, 32, 0, st>>>(code, d);
    g_launch_count += 1;
    cudaError_t ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(out, d, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    cudaFree(d);
    return ce == cudaSuccess ? 0 : 3;
}

extern "C" int orth_gb300_poison_shared_memory(unsigned long long bits, void* stream) {
    using namespace bcgs;
    int dev = 0, sms = 0, smem = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 3;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 3;
    if (cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 3;
    if (cudaFuncSetAttribute(fill_shared_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return 3;
    // One CTA per SM at a time (it takes all of the opt-in shared memory); several
    // waves so that every SM runs at least one.
    fill_shared_kernel<<<(unsigned)(4 * sms), 256, (size_t)smem, (cudaStream_t)stream>>>(bits, smem / 8);
    g_launch_count += 1;
    return cudaGetLastError() == cudaSuccess ? 0 : 3;
}
