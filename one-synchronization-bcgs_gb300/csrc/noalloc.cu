// BCGSI+P-1S on device buffers without any device allocation.
//
// Some callers cannot call cudaMalloc at all: code that runs inside another
// framework's memory pool or allocator callback, where a stray cudaMalloc would
// bypass the pool's accounting or synchronize the device at the wrong moment;
// embedded and real-time callers whose memory budget is fixed at start-up; and
// callers whose stack forbids driver allocations after initialization. For them
// this file provides orth_gb300_bcgsi2P1s_dev_noalloc: the same FP64 kernels as
// orth_gb300_run_dev(ORTH_GB300_BCGSI2P1S, ...), with every piece of scratch
// memory (the Gram partial sums, the small s x s and K x s blocks, the status
// words and the TSQR tree) carved from one fixed device array that is part of
// the loaded library.
//
// Limits and sharing:
//   * The array holds kNoAllocBytes (16 MiB) on every GPU that loads the
//     library, until the process exits. A shape whose scratch does not fit is
//     rejected with ORTH_GB300_NOALLOC_TOO_LARGE and a message on stderr; for
//     example m up to 2^19 rows with n up to 512 and s up to 16 fits.
//   * Every call uses the same array, and the array keeps what the last call
//     left in it. Calls whose work overlaps on the GPU (two streams, or two host
//     threads) race on it; issue them one after another.
//   * The first call on a device looks up the device address of the array
//     (cudaGetSymbolAddress, with that device current), and the launchers raise
//     the shared-memory limits of the kernels it launches on that device (they
//     record this per device and per kernel). Make that first call on each
//     device before any stream capture.
#include <cstdio>
#include <mutex>

#include "../../include/orth_gb300.h"
#include "common.cuh"
#include "kernels.h"

namespace bcgs {
namespace {

constexpr size_t kNoAllocBytes = (size_t)16 << 20;
constexpr size_t kNoAllocDoubles = kNoAllocBytes / sizeof(double);
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

struct DeviceSetup {
    double* scratch = nullptr;  // device address of g_noalloc_scratch
    int num_sms = kNumSMsDefault;
    bool ready = false;
};
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

// Once per device, with that device current: resolve the array's device
// address. In host code the symbol names a host-side shadow, not device memory.
int setup_device(DeviceSetup** out) {
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return (int)ce;
    if (dev < 0 || dev >= kMaxDevices) return (int)cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup& d = g_setup[dev];
    if (!d.ready) {
        void* p = nullptr;
        ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (ce != cudaSuccess) return (int)ce;
        ce = cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (ce != cudaSuccess) return (int)ce;
        d.scratch = static_cast<double*>(p);
        d.ready = true;
    }
    *out = &d;
    return 0;
}

// Scratch layout (doubles), all offsets rounded to 32 doubles (256 bytes).
struct Layout {
    i64 status, G1, G2, Scol, Sd, Yd, part, tsqr, total;
};

i64 round32(i64 v) { return (v + 31) / 32 * 32; }

Layout layout_for(i64 m, int n, int s, int num_sms) {
    i64 part = 0;
    for (int na = 1; na <= n + s; ++na)
        for (int nb = 1; nb <= 2 * s; ++nb) {
            i64 v = gram_chunks_fp64(m, na, nb, num_sms) * (i64)na * nb;
            if (v > part) part = v;
        }
    Layout L;
    i64 off = 0;
    L.status = off; off += 32;                                   // 4 int32 status words
    L.G1 = off;     off += round32((i64)(n + s) * 2 * s);
    L.G2 = off;     off += round32((i64)(n + s) * 2 * s);
    L.Scol = off;   off += round32((i64)n * s);
    L.Sd = off;     off += round32((i64)s * s);
    L.Yd = off;     off += round32((i64)s * s);
    L.part = off;   off += round32(part);
    L.tsqr = off;   off += round32(tsqr_workspace_doubles(m, s));
    L.total = off;
    return L;
}

}  // namespace
}  // namespace bcgs

using namespace bcgs;

extern "C" int orth_gb300_bcgsi2P1s_dev_noalloc(int m, int n, int s, double* dX, long long ldX,
                                                double* dR, int ldR, void* stream,
                                                orth_gb300_status* status) {
    if (status) { status->breakdown_step = 0; status->breakdown_info = 0; status->timeout = 0; status->cuda_error = 0; }
    if (m < 1 || s < 1 || s > 64 || n < 2 * s || ldX < m || ldR < n || (i64)m < n || !dX || !dR)
        return 2;
    DeviceSetup* d = nullptr;
    int rc = setup_device(&d);
    if (rc) {
        if (status) status->cuda_error = rc;
        return 3;
    }
    const Layout L = layout_for(m, n, s, d->num_sms);
    if ((size_t)L.total > kNoAllocDoubles) {
        fprintf(stderr,
                "orth_gb300_bcgsi2P1s_dev_noalloc: m=%d n=%d s=%d needs %lld bytes of scratch; "
                "the static workspace holds %zu bytes\n",
                m, n, s, (long long)L.total * 8, kNoAllocBytes);
        return ORTH_GB300_NOALLOC_TOO_LARGE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    double* base = d->scratch;
    int* stat = reinterpret_cast<int*>(base + L.status);
    double* G1 = base + L.G1;
    double* W = base + L.G2;
    double* Scol = base + L.Scol;
    double* Sd = base + L.Sd;
    double* Yd = base + L.Yd;
    double* part = base + L.part;
    double* tws = base + L.tsqr;
    const i64 M = m, ld = ldX;

    // The status words must start at zero (the array keeps the last call's
    // contents); everything else is written before it is read. A kernel clears
    // them, so the clear does not queue behind copy-engine work on the stream.
    int err = zero_async(stat, kStatusWords * sizeof(int), st);
    auto gram = [&](int na, int b0, int nb, double* C) {
        if (err) return;
        err = launch_gram_fp64(dX, ld, M, 0, na, b0, nb, C, na, part,
                               gram_chunks_fp64(M, na, nb, d->num_sms), st);
    };
    auto update = [&](int K, int c0, int nc, const double* S, int lds, const double* T, int ldt) {
        if (!err) err = launch_update_fp64(dX, ld, M, 0, K, c0, nc, S, lds, T, ldt, st);
    };
    auto pchol = [&](const double* Om, int ldom, const double* A, int lda, int k, int nz, double* T,
                     int step) {
        if (!err) err = launch_pyth_chol(Om, ldom, A, lda, k, nz, T, nz, stat, step, st);
    };

    // BCGSI+P-1S, the same schedule as the allocating entry point
    // (reference SRC/orth.c:48-222).
    const int s0 = s, p = (n - s + s - 1) / s;
    if (!err) err = launch_tsqr(dX, ld, M, 0, s0, dR, ldR, tws, st);
    gram(2 * s, s0, s, W);
    pchol(W + s0, 2 * s, W, 2 * s, s0, s, Sd, 1);
    update(s0, s0, s, W, 2 * s, Sd, s);
    int nZ = n - s - s0 < s ? n - s - s0 : s;
    int na = 2 * s + nZ, nb = s + nZ;
    double* G = G1;
    gram(na, s0, nb, G);
    pchol(G + s0, na, G, na, s0, s, Yd, 1);
    update(s0, s0, s, G, na, Yd, s);
    if (!err) err = launch_rblock(dR, ldR, s0, s0, s, W, 2 * s, G, na, Sd, s, Yd, s, 0, st);
    int ldg = na, mZ = s0;
    for (int i = 1; i < p; ++i) {
        const int mScol = mZ + s;
        if (!err) err = launch_scol(G, ldg, mZ, s, nZ, Yd, s, Scol, mScol, st);
        pchol(G + mScol + (i64)s * ldg, ldg, Scol, mScol, mScol, nZ, Sd, i + 1);
        update(mScol, mScol, nZ, Scol, mScol, Sd, nZ);
        int nY, nZn;
        if (i < p - 1) {
            nZn = n - (i + 1) * s - s0 < s ? n - (i + 1) * s - s0 : s;
            na = mScol + s + nZn;
            nb = s + nZn;
            nY = s;
        } else {
            nZn = nZ;
            na = mScol + nZ;
            nb = nZ;
            nY = nZ;
        }
        gram(na, mScol, nb, G);
        ldg = na;
        pchol(G + mScol, ldg, G, ldg, mScol, nY, Yd, i + 1);
        update(mScol, mScol, nY, G, ldg, Yd, nY);
        if (!err) err = launch_rblock(dR, ldR, mScol, mScol, nY, Scol, mScol, G, ldg, Sd, nY, Yd, nY, 0, st);
        mZ += s;
        nZ = nZn;
    }
    if (status) {
        int h[kStatusWords] = {0, 0, 0, 0};
        if (!err) {
            err = (int)cudaMemcpyAsync(h, stat, sizeof(h), cudaMemcpyDeviceToHost, st);
            if (!err) err = (int)cudaStreamSynchronize(st);
        }
        status->breakdown_step = h[0];
        status->breakdown_info = h[1];
        status->timeout = h[2];
        status->cuda_error = err;
    }
    return err ? 3 : 0;
}
