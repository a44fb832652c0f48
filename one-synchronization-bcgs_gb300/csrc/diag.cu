// Diagnostics: fill every SM's shared memory with one bit pattern.
//
// A kernel that reads shared memory it did not write sees whatever an earlier CTA
// on that SM left there: harmless leftovers in one run, NaN bit patterns from
// another stream's kernel in the next. Filling shared memory with NaN before a
// run makes such reads show up deterministically (tests/test_stale_smem_gpu.py).
#include "../../include/orth_gb300.h"
#include "common.cuh"
#include "kernels.h"

namespace bcgs {

__global__ void fill_shared_kernel(unsigned long long bits, int words) {
    extern __shared__ unsigned long long sfill[];
    for (int i = threadIdx.x; i < words; i += blockDim.x) sfill[i] = bits;
    __syncthreads();
}

}  // namespace bcgs

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
