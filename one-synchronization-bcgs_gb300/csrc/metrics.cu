// Accuracy metrics of a finished QR on the device: the GPU form of the reference's
// test_orth_accuracy (SRC/util.c:36-75), which prints
//   loss of orthogonality  ||Q^T Q - I||_F   (dgemm 'T','N' + allreduce + dnrm2, :50-58)
//   backward error         ||Q R - X||_F     (dlacpy + dgemm 'N','N' + dnrm2, :60-72).
//
// Both sums of squares are accumulated in double-double (TwoSum/TwoProduct with
// FMA) in a fixed order, so the norms are correct to about one unit in the last
// place of FP64 and bit-identical run to run. The Gram Q^T Q itself comes from
// either the FP64 Gram kernel or the exact-accumulation tensor-core digit Gram
// (chosen by the caller); only its upper triangle is formed and mirrored, so the
// error matrix E = Q^T Q - I handed back for the 2-norm is exactly symmetric.
#include "common.cuh"
#include "kernels.h"

namespace bcgs {

namespace {

struct DD {
    double hi, lo;
};

// Knuth's TwoSum: s + e = a + b exactly.
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Accumulate v (with an optional exact low part vlo) into the double-double acc.
__device__ __forceinline__ void dd_add(DD& acc, double v, double vlo) {
    double s, e;
    two_sum(acc.hi, v, s, e);
    acc.hi = s;
    acc.lo += e + vlo;
}

// a + b for double-doubles, renormalized.
__device__ __forceinline__ DD dd_plus(DD a, DD b) {
    double s, e;
    two_sum(a.hi, b.hi, s, e);
    e += a.lo + b.lo;
    DD r;
    r.hi = s + e;
    r.lo = e - (r.hi - s);
    return r;
}

// x^2 added exactly (TwoProduct by FMA) into acc.
__device__ __forceinline__ void dd_add_sq(DD& acc, double x) {
    const double p = x * x;
    const double e = fma(x, x, -p);
    dd_add(acc, p, e);
}

// Fixed-order CTA reduction of one double-double per thread (blockDim.x a multiple
// of 32, <= 1024). Thread 0 returns the total.
__device__ DD block_sum_dd(DD v) {
    __shared__ double sh[32], sl[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        DD w;
        w.hi = __shfl_down_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_down_sync(0xffffffffu, v.lo, o);
        if (lane < o) v = dd_plus(v, w);
    }
    if (lane == 0) { sh[warp] = v.hi; sl[warp] = v.lo; }
    __syncthreads();
    DD t = {0.0, 0.0};
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        for (int w = 0; w < nw; ++w) t = dd_plus(t, DD{sh[w], sl[w]});
    }
    __syncthreads();
    return t;
}

constexpr int RS_THREADS = 128;   // rows per residual tile (one per thread)
constexpr int RS_NC = 32;         // columns per residual group
constexpr int RS_KCH = 32;        // rows of R staged per shared-memory chunk
constexpr int RS_MAX_GRID = 1024; // CTAs per column group

}  // namespace

// E = G - I over the upper triangle of G (n x n, ld ldg), mirrored to the lower one;
// out[0] = ||E||_F. One CTA; entries are visited in a fixed thread assignment and
// reduced in a fixed order.
__global__ void __launch_bounds__(1024)
loo_finish_kernel(const double* __restrict__ G, int ldg, int n, double* __restrict__ E, int lde,
                  double* __restrict__ out) {
    DD acc = {0.0, 0.0};
    const i64 total = (i64)n * n;
    for (i64 e = threadIdx.x; e < total; e += blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        if (i > j) continue;
        double v = G[i + (i64)j * ldg];
        if (i == j) v -= 1.0;
        E[i + (i64)j * lde] = v;
        E[j + (i64)i * lde] = v;
        if (i == j) dd_add_sq(acc, v);
        else { dd_add_sq(acc, v); dd_add_sq(acc, v); }
    }
    const DD t = block_sum_dd(acc);
    if (threadIdx.x == 0) out[0] = sqrt(t.hi + t.lo);
}

// Residual partials. Column group blockIdx.y covers columns [c0, c0+32); CTA bx
// walks the 128-row tiles bx, bx + gridDim.x, ... For each row r and column j,
//   d = sum_{k <= j} Q[r, k] R[k, j] - X[r, j]   (FMA chain in k order; R upper)
// and d^2 and X[r, j]^2 go into per-thread double-doubles.
// part[(group * gridDim.x + bx) * 4 + {0,1,2,3}] = {res.hi, res.lo, x.hi, x.lo}.
__global__ void __launch_bounds__(RS_THREADS)
resid_partial_kernel(const double* __restrict__ X, i64 ldx, const double* __restrict__ Q, i64 ldq, i64 m,
                     int n, const double* __restrict__ R, int ldr, double* __restrict__ part) {
    __shared__ double sR[RS_KCH][RS_NC];
    const int c0 = blockIdx.y * RS_NC;
    const int nc = min(RS_NC, n - c0);
    const int K = c0 + nc;   // R[k, j] = 0 for k > j
    const i64 ntiles = ceil_div(m, RS_THREADS);
    DD res = {0.0, 0.0}, xs = {0.0, 0.0};
    for (i64 tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const i64 r = tile * RS_THREADS + threadIdx.x;
        const bool live = r < m;
        double acc[RS_NC];
#pragma unroll
        for (int j = 0; j < RS_NC; ++j) acc[j] = 0.0;
        for (int k0 = 0; k0 < K; k0 += RS_KCH) {
            const int kc = min(RS_KCH, K - k0);
            __syncthreads();
            for (int e = threadIdx.x; e < RS_KCH * RS_NC; e += RS_THREADS) {
                const int kk = e / RS_NC, j = e % RS_NC;
                const int k = k0 + kk;
                sR[kk][j] = (kk < kc && j < nc && k <= c0 + j) ? R[k + (i64)(c0 + j) * ldr] : 0.0;
            }
            __syncthreads();
            if (live) {
                const double* qr = Q + r + (i64)k0 * ldq;
#pragma unroll 4
                for (int kk = 0; kk < kc; ++kk) {
                    const double q = qr[(i64)kk * ldq];
#pragma unroll
                    for (int j = 0; j < RS_NC; ++j) acc[j] = fma(q, sR[kk][j], acc[j]);
                }
            }
        }
        if (live) {
            const double* xr = X + r + (i64)c0 * ldx;
#pragma unroll
            for (int j = 0; j < RS_NC; ++j) {
                if (j < nc) {
                    const double x = xr[(i64)j * ldx];
                    dd_add_sq(res, acc[j] - x);
                    dd_add_sq(xs, x);
                }
            }
        }
    }
    const DD tr = block_sum_dd(res);
    const DD tx = block_sum_dd(xs);
    if (threadIdx.x == 0) {
        double* o = part + ((i64)blockIdx.y * gridDim.x + blockIdx.x) * 4;
        o[0] = tr.hi; o[1] = tr.lo; o[2] = tx.hi; o[3] = tx.lo;
    }
}

// Sequential fixed-order sum of the partials: out[1] = ||QR - X||_F, out[2] = ||X||_F.
__global__ void resid_finish_kernel(const double* __restrict__ part, int count, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    DD r = {0.0, 0.0}, x = {0.0, 0.0};
    for (int i = 0; i < count; ++i) {
        r = dd_plus(r, DD{part[4 * i], part[4 * i + 1]});
        x = dd_plus(x, DD{part[4 * i + 2], part[4 * i + 3]});
    }
    out[1] = sqrt(r.hi + r.lo);
    out[2] = sqrt(x.hi + x.lo);
}

int metrics_resid_grid(i64 m) {
    const i64 ntiles = ceil_div(m, RS_THREADS);
    return (int)(ntiles < RS_MAX_GRID ? ntiles : RS_MAX_GRID);
}

i64 metrics_part_doubles(i64 m, int n) {
    return (i64)metrics_resid_grid(m) * ceil_div(n, RS_NC) * 4;
}

int launch_loo_finish(const double* G, int ldg, int n, double* E, int lde, double* out, cudaStream_t st) {
    if (n <= 0) return 0;
    loo_finish_kernel<<<1, 1024, 0, st>>>(G, ldg, n, E, lde, out);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

int launch_residual(const double* X, i64 ldx, const double* Q, i64 ldq, i64 m, int n, const double* R, int ldr,
                    double* part, double* out, cudaStream_t st) {
    if (n <= 0 || m <= 0) return 0;
    const int gx = metrics_resid_grid(m);
    const int gy = (int)ceil_div(n, RS_NC);
    resid_partial_kernel<<<dim3((unsigned)gx, (unsigned)gy), RS_THREADS, 0, st>>>(X, ldx, Q, ldq, m, n, R, ldr,
                                                                                   part);
    resid_finish_kernel<<<1, 32, 0, st>>>(part, gx * gy, out);
    g_launch_count += 2;
    return (int)cudaGetLastError();
}

}  // namespace bcgs
