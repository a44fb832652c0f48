// FP64 pipe throughput probe: the roofline denominator of the plain-FP64 form.
// Independent DFMA chains per thread, enough CTAs to fill every SM; reports
// FLOP/s (2 per DFMA) from CUDA events around one launch after a warm-up launch.
#include "common.cuh"
#include "kernels.h"

namespace bcgs {

__global__ void dfma_probe_kernel(double* out, int iters, double a, double b) {
    double acc[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] = (double)(threadIdx.x + c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[c] = fma(acc[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += acc[c];
    if (s == -1.2345) out[0] = s;  // keeps the chains live; never true in practice
}

}  // namespace bcgs

extern "C" int orth_gb300_fp64_peak_probe(double* tflops) {
    using namespace bcgs;
    int dev = 0, sms = kNumSMsDefault;
    BCGS_CUDA_TRY(cudaGetDevice(&dev));
    BCGS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* out = nullptr;
    BCGS_CUDA_TRY(cudaMalloc(&out, sizeof(double)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = 4 * sms, threads = 256, iters = 20000;
    dfma_probe_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e0);
    dfma_probe_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaError_t ce = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (ce != cudaSuccess) return (int)ce;
    const double flops = 2.0 * blocks * threads * (double)iters * 8.0;
    if (tflops) *tflops = flops / (ms * 1e-3) / 1e12;
    return 0;
}
