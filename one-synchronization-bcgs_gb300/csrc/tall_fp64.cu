// Plain-FP64 tall kernels of the BCGS hot path.
//
// On GB300 the FP64 pipe delivers about 1.2 TFLOP/s (two DFMA per SM per clock),
// while the tall products carry about 16 FLOP per byte of HBM traffic, so every
// kernel in this file is bound by the FP64 pipe, not by HBM. The kernels are
// therefore shaped to keep the DFMA pipe fed with few other instructions per
// DFMA, and to reduce deterministically.
//
//   gram_fp64_partial  + gram_reduce : C = X[:, a0:a0+na]^T X[:, b0:b0+nb]
//       replaces the reference's dgemm('T','N') + MPI_Allreduce pair
//       (e.g. SRC/orth.c:182-188). One "synchronization" = one partial pass plus
//       one fixed-order reduction.
//   update_fp64 : Xc = (Xc - X[:, 0:K] S) T^{-1}, T upper triangular
//       replaces dgemm('N','N') + dtrsm('R','U','N','N') (SRC/orth.c:173-176).
#include "common.cuh"
#include "kernels.h"

namespace bcgs {

// ---------------------------------------------------------------------------
// Gram partials. CTA tile: 64 rows of C (columns of A) x 32 columns of C
// (columns of B). 256 threads, each owning a 4 x 2 register tile. The CTA walks a
// contiguous row range of X in sub-tiles of 32 rows staged in shared memory.
// Partial sums go to part[chunk][i + j * na] (column-major na x nb per chunk).
// ---------------------------------------------------------------------------
namespace {
constexpr int GT_A = 64;    // C rows per CTA
constexpr int GT_B = 32;    // C columns per CTA
constexpr int GT_R = 32;    // X rows per shared-memory sub-tile
constexpr int GT_THREADS = 256;
}  // namespace

__global__ void __launch_bounds__(GT_THREADS)
gram_fp64_partial(const double* __restrict__ X, i64 ld, i64 m, int a0, int na, int b0, int nb,
                  i64 rows_per_chunk, double* __restrict__ part) {
    __shared__ double sA[GT_R][GT_A + 1];
    __shared__ double sB[GT_R][GT_B + 1];
    const int chunk = blockIdx.x;
    const int ia0 = blockIdx.y * GT_A;
    const int jb0 = blockIdx.z * GT_B;
    const i64 r_begin = (i64)chunk * rows_per_chunk;
    const i64 r_end = min(m, r_begin + rows_per_chunk);
    const int tid = threadIdx.x;
    const int ti = tid % 16;   // 16 threads along C rows  -> 4 rows each
    const int tj = tid / 16;   // 16 threads along C cols  -> 2 cols each

    double acc[4][2];
#pragma unroll
    for (int a = 0; a < 4; ++a) { acc[a][0] = 0.0; acc[a][1] = 0.0; }

    for (i64 r0 = r_begin; r0 < r_end; r0 += GT_R) {
        // Stage A[r0:r0+32, ia0:ia0+64] and B[r0:r0+32, jb0:jb0+32]. Consecutive
        // threads read consecutive rows of one column: coalesced 256-byte runs.
        for (int e = tid; e < GT_R * GT_A; e += GT_THREADS) {
            int rr = e % GT_R, cc = e / GT_R;
            i64 r = r0 + rr;
            int c = ia0 + cc;
            sA[rr][cc] = (r < r_end && c < na) ? X[r + (i64)(a0 + c) * ld] : 0.0;
        }
        for (int e = tid; e < GT_R * GT_B; e += GT_THREADS) {
            int rr = e % GT_R, cc = e / GT_R;
            i64 r = r0 + rr;
            int c = jb0 + cc;
            sB[rr][cc] = (r < r_end && c < nb) ? X[r + (i64)(b0 + c) * ld] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int rr = 0; rr < GT_R; ++rr) {
            double av[4], bv[2];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = sA[rr][ti + 16 * a];
            bv[0] = sB[rr][tj];
            bv[1] = sB[rr][tj + 16];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                acc[a][0] = fma(av[a], bv[0], acc[a][0]);
                acc[a][1] = fma(av[a], bv[1], acc[a][1]);
            }
        }
        __syncthreads();
    }
    double* out = part + (i64)chunk * na * nb;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        int i = ia0 + ti + 16 * a;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            int j = jb0 + tj + 16 * b;
            if (i < na && j < nb) out[i + (i64)j * na] = acc[a][b];
        }
    }
}

// Fixed-order sum over chunks: out[i + j*ldo] = sum_{c=0}^{nchunks-1} part[c][i + j*na].
// Each entry is summed sequentially in chunk order, so results are bit-identical
// run to run for a given (m, na, nb).
__global__ void gram_reduce(const double* __restrict__ part, int nchunks, int na, int nb,
                            double* __restrict__ out, int ldo) {
    const i64 total = (i64)na * nb;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total;
         e += (i64)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < nchunks; ++c) s += part[(i64)c * total + e];
        int i = (int)(e % na), j = (int)(e / na);
        out[i + (i64)j * ldo] = s;
    }
}

int gram_chunks_fp64(i64 m, int na, int nb, int num_sms) {
    const i64 tiles = ceil_div(na, GT_A) * ceil_div(nb, GT_B);
    // About four CTAs per SM in total, each with at least 256 rows.
    i64 want = ceil_div(4LL * num_sms, tiles);
    i64 max_by_rows = ceil_div(m, 256);
    i64 c = want < max_by_rows ? want : max_by_rows;
    if (c < 1) c = 1;
    if (c > 4096) c = 4096;
    return (int)c;
}

int launch_gram_fp64(const double* X, i64 ld, i64 m, int a0, int na, int b0, int nb,
                     double* out, int ldo, double* part, int nchunks, cudaStream_t st) {
    if (na <= 0 || nb <= 0) return 0;
    i64 rows_per_chunk = ceil_div(m, nchunks);
    rows_per_chunk = ceil_div(rows_per_chunk, GT_R) * GT_R;
    dim3 grid((unsigned)nchunks, (unsigned)ceil_div(na, GT_A), (unsigned)ceil_div(nb, GT_B));
    gram_fp64_partial<<<grid, GT_THREADS, 0, st>>>(X, ld, m, a0, na, b0, nb, rows_per_chunk, part);
    i64 total = (i64)na * nb;
    int blocks = (int)ceil_div(total, 256);
    if (blocks > 4 * 152) blocks = 4 * 152;
    gram_reduce<<<blocks, 256, 0, st>>>(part, nchunks, na, nb, out, ldo);
    g_launch_count += 2;
    return (int)cudaGetLastError();
}

int launch_gram_reduce(const double* part, int nchunks, int na, int nb, double* out, int ldo,
                       cudaStream_t st) {
    const i64 total = (i64)na * nb;
    int blocks = (int)ceil_div(total, 256);
    if (blocks > 4 * 152) blocks = 4 * 152;
    gram_reduce<<<blocks, 256, 0, st>>>(part, nchunks, na, nb, out, ldo);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Update: Xc[r, 0:nc] = (Xc[r, :] - sum_c Q[r, c] S[c, :]) * T^{-1}.
// One thread per row with NC register accumulators; S is staged through shared
// memory in chunks of 64 rows (broadcast reads). T is upper triangular (nc x nc,
// ld ldt); its diagonal is inverted once per CTA. If T is null the scaling is
// skipped (bcgsi21s's unscaled first pass, SRC/orth.c:323-324).
// ---------------------------------------------------------------------------
namespace {
constexpr int UP_THREADS = 128;
}  // namespace

// Rows of S staged per shared-memory chunk; keeps static shared memory < 48 KB.
template <int NC>
struct UpChunk { static constexpr int value = NC <= 16 ? 64 : (NC <= 32 ? 32 : 16); };

template <int NC>
__global__ void __launch_bounds__(UP_THREADS)
update_fp64(double* __restrict__ X, i64 ld, i64 m, int q0, int K, int c0, int nc,
            const double* __restrict__ S, int lds, const double* __restrict__ T, int ldt) {
    constexpr int KCH = UpChunk<NC>::value;
    __shared__ double sS[KCH][NC];
    __shared__ double sT[NC][NC];
    __shared__ double sRd[NC];
    const int tid = threadIdx.x;
    const i64 r = blockIdx.x * (i64)UP_THREADS + tid;
    if (T != nullptr) {
        for (int e = tid; e < NC * NC; e += UP_THREADS) {
            int i = e % NC, j = e / NC;
            sT[i][j] = (i < nc && j < nc && i <= j) ? T[i + (i64)j * ldt] : 0.0;
        }
    }
    __syncthreads();
    if (T != nullptr && tid < NC) sRd[tid] = (tid < nc) ? 1.0 / sT[tid][tid] : 0.0;

    double acc[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) acc[j] = 0.0;
    const bool live = r < m;
    for (int k0 = 0; k0 < K; k0 += KCH) {
        const int kc = min(KCH, K - k0);
        __syncthreads();
        for (int e = tid; e < KCH * NC; e += UP_THREADS) {
            int kk = e / NC, j = e % NC;
            sS[kk][j] = (kk < kc && j < nc) ? S[(k0 + kk) + (i64)j * lds] : 0.0;
        }
        __syncthreads();
        if (live) {
            const double* qrow = X + r + (i64)(q0 + k0) * ld;
#pragma unroll 4
            for (int kk = 0; kk < kc; ++kk) {
                const double q = qrow[(i64)kk * ld];
#pragma unroll
                for (int j = 0; j < NC; ++j) acc[j] = fma(q, sS[kk][j], acc[j]);
            }
        }
    }
    __syncthreads();
    if (!live) return;
    double* xr = X + r + (i64)c0 * ld;
    // acc becomes w = x - Q S in place.
#pragma unroll
    for (int j = 0; j < NC; ++j) acc[j] = (j < nc) ? xr[(i64)j * ld] - acc[j] : 0.0;
    if (T != nullptr) {
        // Forward substitution u T = w (dtrsm 'R','U','N','N'), column by column.
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            double v = acc[j];
#pragma unroll
            for (int i = 0; i < j; ++i) v = fma(-acc[i], sT[i][j], v);
            acc[j] = v * sRd[j];
        }
    }
#pragma unroll
    for (int j = 0; j < NC; ++j)
        if (j < nc) xr[(i64)j * ld] = acc[j];
}

int launch_update_fp64(double* X, i64 ld, i64 m, int q0, int K, int c0, int nc,
                       const double* S, int lds, const double* T, int ldt, cudaStream_t st) {
    if (nc <= 0 || m <= 0) return 0;
    dim3 grid((unsigned)ceil_div(m, UP_THREADS));
    if (nc <= 8)
        update_fp64<8><<<grid, UP_THREADS, 0, st>>>(X, ld, m, q0, K, c0, nc, S, lds, T, ldt);
    else if (nc <= 16)
        update_fp64<16><<<grid, UP_THREADS, 0, st>>>(X, ld, m, q0, K, c0, nc, S, lds, T, ldt);
    else if (nc <= 32)
        update_fp64<32><<<grid, UP_THREADS, 0, st>>>(X, ld, m, q0, K, c0, nc, S, lds, T, ldt);
    else if (nc <= 64)
        update_fp64<64><<<grid, UP_THREADS, 0, st>>>(X, ld, m, q0, K, c0, nc, S, lds, T, ldt);
    else
        return (int)cudaErrorInvalidValue;
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

}  // namespace bcgs
