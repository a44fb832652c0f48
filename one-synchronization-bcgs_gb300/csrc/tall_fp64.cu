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
#include "batched.h"
#include "common.cuh"
#include "kernels.h"

namespace bcgs {

namespace {
// Single-matrix Gram: one CTA per 16-column strip of A x 32 columns of B x row
// chunk, so na (a multiple of s) wastes no work on zero padding.
constexpr int GS_A = 16;            // C rows per CTA
constexpr int GS_B = 32;            // C columns per CTA
constexpr int GS_R = 16;            // X rows per shared-memory sub-tile
constexpr int GS_CTAS_PER_SM = 16;  // resident strip CTAs per SM (64 registers, 7 KB)
constexpr int GT_R = 32;            // chunk row ranges are multiples of this
}  // namespace

// ---------------------------------------------------------------------------
// Gram partials. CTA tile: GA rows of C (columns of A) x TB columns of C (columns
// of B); (GA/4) x (TB/2) threads, each owning a 4 x 2 register tile. The CTA walks
// a contiguous row range of X in sub-tiles of GR rows staged in shared memory.
// Partial sums go to part[chunk][i + j * na] (column-major na x nb per chunk).
// Every entry is a sequential FMA chain over the rows of the chunk in order, so
// the result depends on the chunking only, not on GA, TB or GR.
// ---------------------------------------------------------------------------
template <int GA_, int TB_, int GR_>
struct GramTile {
    static constexpr int GA = GA_, TB = TB_, GR = GR_;
    static constexpr int NT = (GA / 4) * (TB / 2);                // threads
    static constexpr int SMEM = GR * (GA + 1) + GR * (TB + 1);    // doubles
};
// Batched form: 64 threads, GA = 512 / TB, TB in {8, 16, 32} (B panels of 2s
// columns for s = 4, 8, 16 against A strips of 64, 32 or 16 columns).
template <int TB>
using GramPanel = GramTile<512 / TB, TB, 16>;
using GramStrip = GramTile<GS_A, GS_B, GS_R>;
static_assert(GramStrip::NT == 64 && GramPanel<8>::NT == 64 && GramPanel<16>::NT == 64 && GramPanel<32>::NT == 64,
              "strip CTAs are two warps");
constexpr int kGramSmemMax = GramPanel<32>::SMEM > GramPanel<8>::SMEM
                                 ? (GramPanel<32>::SMEM > GramPanel<16>::SMEM ? GramPanel<32>::SMEM
                                                                              : GramPanel<16>::SMEM)
                                 : (GramPanel<8>::SMEM > GramPanel<16>::SMEM ? GramPanel<8>::SMEM
                                                                             : GramPanel<16>::SMEM);

// The tile at C rows ia0.., C columns jb0.., rows [r_begin, r_end) of X, written to
// `out` (na x nb, ld na). Tile::NT threads; sm holds Tile::SMEM doubles.
// SEGR > 0: every SEGR rows the running sums are added to a total and restarted,
// so no FMA chain is longer than SEGR rows however long the row range is
// (SEGR = 0: one chain over the range).
template <class Tile, int SEGR = 0>
__device__ __forceinline__ void gram_partial_body(const double* __restrict__ X, i64 ld, int a0, int na, int b0,
                                                  int nb, i64 r_begin, i64 r_end, int ia0, int jb0,
                                                  double* __restrict__ out, double* __restrict__ sm) {
    constexpr int GA = Tile::GA, TB = Tile::TB, GR = Tile::GR, NT = Tile::NT;
    constexpr int SEG = SEGR / GR;  // sub-tiles per segment
    static_assert(SEGR % GR == 0, "segments are whole sub-tiles");
    constexpr int TI = GA / 4;      // threads along C rows -> 4 rows each
    double (*sA)[GA + 1] = reinterpret_cast<double (*)[GA + 1]>(sm);
    double (*sB)[TB + 1] = reinterpret_cast<double (*)[TB + 1]>(sm + GR * (GA + 1));
    const int tid = threadIdx.x;
    const int ti = tid % TI;
    const int tj = tid / TI;        // TB/2 threads along C cols -> 2 cols each

    double acc[4][2], tot[4][2];
#pragma unroll
    for (int a = 0; a < 4; ++a) { acc[a][0] = 0.0; acc[a][1] = 0.0; tot[a][0] = 0.0; tot[a][1] = 0.0; }

    int sub = 0;
    for (i64 r0 = r_begin; r0 < r_end; r0 += GR) {
        if (SEG > 0 && sub == SEG) {
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                tot[a][0] += acc[a][0]; tot[a][1] += acc[a][1];
                acc[a][0] = 0.0; acc[a][1] = 0.0;
            }
            sub = 0;
        }
        ++sub;
        // Stage A[r0:r0+GR, ia0:ia0+GA] and B[r0:r0+GR, jb0:jb0+TB]. Consecutive
        // threads read consecutive rows of one column.
        for (int e = tid; e < GR * GA; e += NT) {
            int rr = e % GR, cc = e / GR;
            i64 r = r0 + rr;
            int c = ia0 + cc;
            sA[rr][cc] = (r < r_end && c < na) ? X[r + (i64)(a0 + c) * ld] : 0.0;
        }
        for (int e = tid; e < GR * TB; e += NT) {
            int rr = e % GR, cc = e / GR;
            i64 r = r0 + rr;
            int c = jb0 + cc;
            sB[rr][cc] = (r < r_end && c < nb) ? X[r + (i64)(b0 + c) * ld] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int rr = 0; rr < GR; ++rr) {
            double av[4], bv[2];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = sA[rr][ti + TI * a];
            bv[0] = sB[rr][tj];
            bv[1] = sB[rr][tj + TB / 2];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                acc[a][0] = fma(av[a], bv[0], acc[a][0]);
                acc[a][1] = fma(av[a], bv[1], acc[a][1]);
            }
        }
        __syncthreads();
    }
    if (SEG > 0) {
#pragma unroll
        for (int a = 0; a < 4; ++a) { acc[a][0] += tot[a][0]; acc[a][1] += tot[a][1]; }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        int i = ia0 + ti + TI * a;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            int j = jb0 + tj + (TB / 2) * b;
            if (i < na && j < nb) out[i + (i64)j * na] = acc[a][b];
        }
    }
}

__global__ void __launch_bounds__(GramStrip::NT, GS_CTAS_PER_SM)
gram_fp64_partial(const double* __restrict__ X, i64 ld, i64 m, int a0, int na, int b0, int nb,
                  i64 rows_per_chunk, double* __restrict__ part) {
    __shared__ double sm[GramStrip::SMEM];
    const int chunk = blockIdx.x;
    const i64 r_begin = (i64)chunk * rows_per_chunk;
    const i64 r_end = min(m, r_begin + rows_per_chunk);
    gram_partial_body<GramStrip>(X, ld, a0, na, b0, nb, r_begin, r_end, blockIdx.y * GS_A, blockIdx.z * GS_B,
                                 part + (i64)chunk * na * nb, sm);
}

// The same over chunks of rows_per_chunk rows, each summed in segments of
// 256 rows (the row-sharded path's long chunks).
__global__ void __launch_bounds__(GramStrip::NT, GS_CTAS_PER_SM)
gram_fp64_partial_seg(const double* __restrict__ X, i64 ld, i64 m, int a0, int na, int b0, int nb,
                      i64 rows_per_chunk, double* __restrict__ part) {
    __shared__ double sm[GramStrip::SMEM];
    const int chunk = blockIdx.x;
    const i64 r_begin = (i64)chunk * rows_per_chunk;
    const i64 r_end = min(m, r_begin + rows_per_chunk);
    gram_partial_body<GramStrip, 256>(X, ld, a0, na, b0, nb, r_begin, r_end, blockIdx.y * GS_A,
                                      blockIdx.z * GS_B, part + (i64)chunk * na * nb, sm);
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

// Rows per Gram chunk forced by orth_gb300_set_gram_chunk_rows (0: the default
// policy below).
long long g_gram_chunk_rows = 0;

int gram_chunks_fp64(i64 m, int na, int nb, int num_sms) {
    if (g_gram_chunk_rows > 0) {
        const i64 c = ceil_div(m, g_gram_chunk_rows);
        return (int)(c < 1 ? 1 : c);
    }
    // One wave: the most chunks whose strip CTAs all fit on the SMs at once, so
    // every SM gets the same number of equal CTAs (within one), each with at
    // least 256 rows. The FP64 pipe is saturated by two resident CTAs per SM;
    // what costs time is an SM holding more CTAs than the others.
    const i64 ctas_per_chunk = ceil_div(na, GS_A) * ceil_div(nb, GS_B);
    i64 want = (i64)GS_CTAS_PER_SM * num_sms / ctas_per_chunk;
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
    dim3 grid((unsigned)nchunks, (unsigned)ceil_div(na, GS_A), (unsigned)ceil_div(nb, GS_B));
    gram_fp64_partial<<<grid, GramStrip::NT, 0, st>>>(X, ld, m, a0, na, b0, nb, rows_per_chunk, part);
    i64 total = (i64)na * nb;
    int blocks = (int)ceil_div(total, 256);
    if (blocks > 4 * 152) blocks = 4 * 152;
    gram_reduce<<<blocks, 256, 0, st>>>(part, nchunks, na, nb, out, ldo);
    g_launch_count += 2;
    g_reduce_count += 1;
    return (int)cudaGetLastError();
}

int launch_gram_partials_fp64(const double* X, i64 ld, i64 m, int a0, int na, int b0, int nb, double* part,
                              i64 rows, cudaStream_t st) {
    if (na <= 0 || nb <= 0 || m <= 0) return 0;
    if (rows <= 0 || rows % GT_R != 0) return (int)cudaErrorInvalidValue;
    const i64 nchunks = ceil_div(m, rows);
    dim3 grid((unsigned)nchunks, (unsigned)ceil_div(na, GS_A), (unsigned)ceil_div(nb, GS_B));
    gram_fp64_partial_seg<<<grid, GramStrip::NT, 0, st>>>(X, ld, m, a0, na, b0, nb, rows, part);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

int launch_gram_reduce(const double* part, int nchunks, int na, int nb, double* out, int ldo,
                       cudaStream_t st) {
    const i64 total = (i64)na * nb;
    int blocks = (int)ceil_div(total, 256);
    if (blocks > 4 * 152) blocks = 4 * 152;
    gram_reduce<<<blocks, 256, 0, st>>>(part, nchunks, na, nb, out, ldo);
    g_launch_count += 1;
    g_reduce_count += 1;
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

// Shared-memory doubles update_body<NC> needs: S chunk, T, T's reciprocal diagonal.
template <int NC>
struct UpSmem { static constexpr int value = UpChunk<NC>::value * NC + NC * NC + NC; };

// Rows [r0, r0 + 128) of the update, one row per thread (128 threads). sm holds
// UpSmem<NC>::value doubles. Every output is an FMA chain over k in order, then the
// forward substitution in column order, so the result does not depend on NC >= nc.
template <int NC>
__device__ __forceinline__ void update_body(double* __restrict__ X, i64 ld, i64 m, int q0, int K, int c0, int nc,
                                            const double* __restrict__ S, int lds, const double* __restrict__ T,
                                            int ldt, i64 r0, double* __restrict__ sm) {
    constexpr int KCH = UpChunk<NC>::value;
    double (*sS)[NC] = reinterpret_cast<double (*)[NC]>(sm);
    double (*sT)[NC] = reinterpret_cast<double (*)[NC]>(sm + KCH * NC);
    double* sRd = sm + KCH * NC + NC * NC;
    const int tid = threadIdx.x;
    const i64 r = r0 + tid;
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
    if (live) {
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
    __syncthreads();   // sm is reused by the caller's next tile
}

template <int NC>
__global__ void __launch_bounds__(UP_THREADS)
update_fp64(double* __restrict__ X, i64 ld, i64 m, int q0, int K, int c0, int nc,
            const double* __restrict__ S, int lds, const double* __restrict__ T, int ldt) {
    __shared__ double sm[UpSmem<NC>::value];
    update_body<NC>(X, ld, m, q0, K, c0, nc, S, lds, T, ldt, blockIdx.x * (i64)UP_THREADS, sm);
}

int launch_update_fp64(double* X, i64 ld, i64 m, int q0, int K, int c0, int nc,
                       const double* S, int lds, const double* T, int ldt, cudaStream_t st) {
    if (nc <= 0 || m <= 0) return 0;
    dim3 grid((unsigned)ceil_div(m, UP_THREADS));
    if (nc <= 4)
        update_fp64<4><<<grid, UP_THREADS, 0, st>>>(X, ld, m, q0, K, c0, nc, S, lds, T, ldt);
    else if (nc <= 8)
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

// ---------------------------------------------------------------------------
// Batched forms: one launch over many matrices' jobs (batched.h).
// ---------------------------------------------------------------------------
int gram_batched_panel_rows(int tb) { return 512 / tb; }

__global__ void __launch_bounds__(64, GS_CTAS_PER_SM)
gram_partial_batched(const GramJob* __restrict__ jobs, const int* __restrict__ prefix, int njobs) {
    __shared__ double sm[kGramSmemMax];
    const int j = batched_job_of(prefix, njobs, blockIdx.x);
    const GramJob& J = jobs[j];
    const int local = blockIdx.x - prefix[j];
    const int chunk = local % J.nchunks;
    const int t = local / J.nchunks;
    const int ia = t % J.tilesA, jb = t / J.tilesA;
    const i64 r_begin = (i64)chunk * J.rows_per_chunk;
    const i64 r_end = min(J.m, r_begin + J.rows_per_chunk);
    double* out = J.part + (i64)chunk * J.na * J.nb;
    const int ia0 = ia * (512 / J.tb);
    if (J.tb == 8)
        gram_partial_body<GramPanel<8>>(J.X, J.ld, 0, J.na, J.b0, J.nb, r_begin, r_end, ia0, jb * 8, out, sm);
    else if (J.tb == 16)
        gram_partial_body<GramPanel<16>>(J.X, J.ld, 0, J.na, J.b0, J.nb, r_begin, r_end, ia0, jb * 16, out, sm);
    else
        gram_partial_body<GramPanel<32>>(J.X, J.ld, 0, J.na, J.b0, J.nb, r_begin, r_end, ia0, jb * 32, out, sm);
}

// Same summation order as gram_reduce: each entry sums the chunks in order.
__global__ void __launch_bounds__(256)
gram_reduce_batched(const GramJob* __restrict__ jobs, const int* __restrict__ prefix, int njobs) {
    const int j = batched_job_of(prefix, njobs, blockIdx.x);
    const GramJob& J = jobs[j];
    const i64 total = (i64)J.na * J.nb;
    const i64 e = (i64)(blockIdx.x - prefix[j]) * 256 + threadIdx.x;
    if (e >= total) return;
    double s = 0.0;
    for (int c = 0; c < J.nchunks; ++c) s += J.part[(i64)c * total + e];
    const int i = (int)(e % J.na), jj = (int)(e / J.na);
    J.C[i + (i64)jj * J.ldc] = s;
}

__global__ void __launch_bounds__(UP_THREADS)
update_batched(const UpdJob* __restrict__ jobs, const int* __restrict__ prefix, int njobs) {
    __shared__ double sm[UpSmem<16>::value];
    const int j = batched_job_of(prefix, njobs, blockIdx.x);
    const UpdJob& J = jobs[j];
    const i64 r0 = (i64)(blockIdx.x - prefix[j]) * UP_THREADS;
    if (J.nc <= 4)
        update_body<4>(J.X, J.ld, J.m, J.q0, J.K, J.c0, J.nc, J.S, J.lds, J.T, J.ldt, r0, sm);
    else if (J.nc <= 8)
        update_body<8>(J.X, J.ld, J.m, J.q0, J.K, J.c0, J.nc, J.S, J.lds, J.T, J.ldt, r0, sm);
    else
        update_body<16>(J.X, J.ld, J.m, J.q0, J.K, J.c0, J.nc, J.S, J.lds, J.T, J.ldt, r0, sm);
}

int launch_gram_partial_batched(const GramJob* jobs, const int* prefix, int njobs, int items, cudaStream_t st) {
    if (items <= 0) return 0;
    gram_partial_batched<<<(unsigned)items, 64, 0, st>>>(jobs, prefix, njobs);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

int launch_gram_reduce_batched(const GramJob* jobs, const int* prefix, int njobs, int items, cudaStream_t st) {
    if (items <= 0) return 0;
    gram_reduce_batched<<<(unsigned)items, 256, 0, st>>>(jobs, prefix, njobs);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

int launch_update_batched(const UpdJob* jobs, const int* prefix, int njobs, int items, cudaStream_t st) {
    if (items <= 0) return 0;
    update_batched<<<(unsigned)items, UP_THREADS, 0, st>>>(jobs, prefix, njobs);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

}  // namespace bcgs
