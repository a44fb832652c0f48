// Internal launcher declarations shared by the kernel files and the C-ABI layer.
// All matrices are column-major FP64 device buffers; every launcher enqueues on
// `st` and returns a cudaError_t value (0 on success).
#pragma once

#include <atomic>

#include <cuda_runtime.h>

namespace bcgs {

using i64 = long long;

// Number of kernels enqueued by the launchers below since load (host counter;
// split-precision batches enqueue from several host threads).
extern std::atomic<long long> g_launch_count;
// Number of launches of the fixed-order Gram reduction (the kernel that stands
// in for each MPI_Allreduce of the reference).
extern std::atomic<long long> g_reduce_count;

// bytes of zeros at p, by a kernel on st (not a copy-engine memset). Counted in
// g_launch_count and also in g_aux_launch_count, which the per-class profile
// subtracts so that its launch counts are those of the classes' own kernels.
int zero_async(void* p, size_t bytes, cudaStream_t st);
extern std::atomic<long long> g_aux_launch_count;

// Raises kernel fn's dynamic shared-memory limit to `bytes` on the current
// device, once per (device, kernel). Call outside any stream capture.
int smem_attr(const void* fn, int bytes);

// C (na x nb, ld ldo) = X[:, a0:a0+na]^T X[:, b0:b0+nb] over m rows, FP64, with a
// fixed-order two-stage reduction through `part` (nchunks * na * nb doubles).
int gram_chunks_fp64(i64 m, int na, int nb, int num_sms);
// Rows per chunk forced by orth_gb300_set_gram_chunk_rows (0: default policy).
extern long long g_gram_chunk_rows;
int launch_gram_fp64(const double* X, i64 ld, i64 m, int a0, int na, int b0, int nb,
                     double* out, int ldo, double* part, int nchunks, cudaStream_t st);

// out (na x nb, ld ldo) = fixed-order sum of nchunks partials part[c][i + j*na].
int launch_gram_reduce(const double* part, int nchunks, int na, int nb, double* out, int ldo,
                       cudaStream_t st);

// X[:, c0:c0+nc] = (X[:, c0:c0+nc] - X[:, q0:q0+K] S) T^{-1}; T upper (nc x nc) or null.
int launch_update_fp64(double* X, i64 ld, i64 m, int q0, int K, int c0, int nc,
                       const double* S, int lds, const double* T, int ldt, cudaStream_t st);

// Small single-CTA kernels (nz, s, ny <= 64).
int launch_pyth_chol(const double* Om, int ldom, const double* A, int lda, int k, int nz,
                     double* T, int ldt, int* status, int step, cudaStream_t st);
int launch_scol(const double* G, int ldg, int mZ, int s, int nZ, const double* Yd, int ldy,
                double* Scol, int ldsc, cudaStream_t st);
int launch_rblock(double* R, int ldR, int c0, int K, int ny, const double* A, int lda,
                  const double* B, int ldb, const double* Sd, int ldsd, const double* Yd,
                  int ldyd, int mode, cudaStream_t st);

// Explicit TSQR of X[:, c0:c0+nc] in place; R (nc x nc, ldR) upper with diag >= 0.
int tsqr_tile_rows(int nc);
i64 tsqr_workspace_doubles(i64 m, int nc);
int launch_tsqr(double* X, i64 ld, i64 m, int c0, int nc, double* R, int ldR, double* ws,
                cudaStream_t st);

// Exchange of the row-sharded path: gathers `count` doubles from every rank into
// `all` (size * count doubles, rank order), ordered on stream st. 0 on success.
typedef int (*ShardGatherFn)(void* ctx, const double* mine, double* all, long long count, cudaStream_t st);

// Row-sharded TSQR of this rank's rows X[0:m_local, c0:c0+nc] (TR-row tiles
// [t0[rank], t0[rank] + nt[rank]) of T). `mine` holds maxt * nc * nc doubles and
// `all` size times that; ws holds tsqr_workspace_doubles(T * TR, nc). R is
// written on every rank.
struct TsqrShard {
    int rank = 0, size = 1;
    i64 T = 0, maxt = 0;
    const i64* t0 = nullptr;   // first tile of each rank
    const i64* nt = nullptr;   // tiles of each rank
    double* mine = nullptr;
    double* all = nullptr;
    ShardGatherFn gather = nullptr;
    void* ctx = nullptr;
};
int launch_tsqr_sharded(double* X, i64 ld, i64 m_local, int c0, int nc, double* R, int ldR, double* ws,
                        const TsqrShard& sh, cudaStream_t st);

// Gram partials only: part[c][i + j*na] = rows [c*rows, (c+1)*rows) of
// X[:, a0:a0+na]^T X[:, b0:b0+nb], for the ceil(m / rows) chunks of exactly
// `rows` rows (a multiple of 32; the last chunk is cut at m). Each chunk is summed
// in segments of 256 rows, so accuracy does not degrade with `rows`.
int launch_gram_partials_fp64(const double* X, i64 ld, i64 m, int a0, int na, int b0, int nb, double* part,
                              i64 rows, cudaStream_t st);

// Accuracy metrics (the reference's test_orth_accuracy, SRC/util.c:36-75).
// E (n x n, lde) = G - I from the upper triangle of the Gram G (ld ldg), mirrored;
// out[0] = ||E||_F (double-double accumulation, fixed order).
int launch_loo_finish(const double* G, int ldg, int n, double* E, int lde, double* out, cudaStream_t st);
// out[1] = ||Q R - X||_F (R upper: entries below its diagonal are not read) and
// out[2] = ||X||_F; part holds metrics_part_doubles(m, n) doubles.
i64 metrics_part_doubles(i64 m, int n);
int launch_residual(const double* X, i64 ldx, const double* Q, i64 ldq, i64 m, int n, const double* R, int ldr,
                    double* part, double* out, cudaStream_t st);

}  // namespace bcgs
