/*
 * Extended C ABI of the GB300 BCGS library: device buffers, a caller stream,
 * a precision mode and a status report. Plain pointers and sizes only.
 *
 * The reference has no counterpart for these entry points; each one runs the
 * same algorithm as the same-named function of include/orth.h (reference
 * include/orth.h:8-17) on buffers that already live on the GPU.
 */
#ifndef ORTH_GB300_H
#define ORTH_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status of the last run. */
typedef struct orth_gb300_status {
    int breakdown_step;  /* 1-based block step of the first Cholesky breakdown, 0 if none */
    int breakdown_info;  /* dpotrf-style info of that breakdown (1-based column) */
    int timeout;         /* a bounded device wait gave up (no kernel here waits on a peer: 0) */
    int cuda_error;      /* cudaError_t of the first failing CUDA call, 0 if none */
} orth_gb300_status;

/*
 * Precision modes of the tall products (Q^T V and Q S). The split modes hold each
 * column as fixed point scaled by the column's maximum, so entries far below
 * their column's maximum keep fewer significant bits than in FP64. The
 * environment variable ORTH_GB300_SPLIT_GRAM_PLANES=6 makes the 56-bit mode's Gram
 * read 6 planes of its first operand (faster, less accurate for columns
 * dominated by a few rows); the default reads all 7.
 */
#define ORTH_GB300_FP64 0             /* plain FP64 on the FP64 pipe */
#define ORTH_GB300_SPLIT_BF16 1       /* tensor cores, 7 BF16 digit planes (56-bit fixed point) */
#define ORTH_GB300_SPLIT_BF16_FAST 2  /* tensor cores, 6 BF16 digit planes (48-bit fixed point) */

/* Variant identifiers for orth_gb300_run_dev. */
#define ORTH_GB300_BCGSI2P1S 0
#define ORTH_GB300_BCGSI21S 1
#define ORTH_GB300_BCGSPIPI2 2
#define ORTH_GB300_BCGSI2 3
#define ORTH_GB300_BCGSI2P2S 4

/*
 * Device-pointer form of the orth.h entry points. dX: m x n column-major FP64
 * on the current device, leading dimension ldX >= m, overwritten with Q.
 * dR: n x n (ldR >= n) device buffer; the upper block triangle is written.
 * stream: a cudaStream_t (NULL = legacy default stream). status: optional; when
 * non-NULL the call waits for the stream and fills it, otherwise the call only
 * enqueues work and returns.
 * Return codes: 0 ok, 2 invalid arguments, 3 CUDA failure, 4 unsupported
 * precision for this variant/shape.
 */
int orth_gb300_run_dev(int variant, int m, int n, int s, double *dX, long long ldX,
                       double *dR, int ldR, int precision, void *stream,
                       orth_gb300_status *status);

/*
 * BCGSI+P-1S on device buffers without allocating. There is no counterpart in
 * the reference. It is for callers that cannot call cudaMalloc: code running
 * inside another framework's memory pool or allocator callback, and embedded or
 * real-time programs whose device memory is fixed at start-up. Arguments and
 * results are those of orth_gb300_run_dev(ORTH_GB300_BCGSI2P1S, ..., FP64).
 * All scratch comes from one 16 MiB array held by the library on every GPU
 * that loads it (for example m up to 2^19 with n <= 512, s <= 16 fits); larger
 * shapes return ORTH_GB300_NOALLOC_TOO_LARGE with a message on stderr. Calls
 * share that array: calls that overlap on the GPU race, so issue them one after
 * another. The first call on a device resolves the array's device address; make
 * it before any stream capture.
 */
#define ORTH_GB300_NOALLOC_TOO_LARGE 5
int orth_gb300_bcgsi2P1s_dev_noalloc(int m, int n, int s, double *dX, long long ldX,
                                     double *dR, int ldR, void *stream,
                                     orth_gb300_status *status);

/*
 * Precision used by the five orth.h entry points (default ORTH_GB300_FP64, the
 * reference's arithmetic; the environment variable ORTH_GB300_PRECISION =
 * fp64 | split | split_fast sets it at first use). Shapes the split modes do not
 * handle (s > 64) return 4. Returns 0, or 4 for an unknown mode.
 */
int orth_gb300_set_host_precision(int precision);

/*
 * Host buffers for the orth.h entry points. Their X and R may be any host
 * memory; page-locked memory lets the copies run while the QR does, and how it
 * was made sets the link rate of long copies. orth_gb300_host_alloc returns (in
 * *ptr) a page-locked buffer of at least `bytes` backed by transparent huge
 * pages where the kernel offers them (an aligned anonymous mapping advised
 * MADV_HUGEPAGE, faulted in, then registered with cudaHostRegister): 32 GiB
 * moved at 210 GB/s to a GB300 and 193 GB/s back, against 81-139 GB/s for
 * cudaHostAlloc memory. A host too fragmented to give huge pages backs such a
 * mapping with base pages (25-34 GB/s); when less than 3/4 of a buffer of 64 MB or
 * more came as huge pages, it is made by cudaHostAlloc instead. The memory reads
 * as zero. Returns 0; 2 for a null ptr or zero bytes; 6 if the mapping fails; 3 if
 * the registration or cudaHostAlloc fails.
 * orth_gb300_host_free releases a buffer from orth_gb300_host_alloc (0; 2 for a
 * pointer it did not return; 3 if the unregistration fails; a null pointer is a
 * no-op).
 * orth_gb300_host_buffer_info reports how a buffer from orth_gb300_host_alloc was
 * made: *kind = 1 (huge-page mapping, registered) or 2 (cudaHostAlloc), and
 * *huge_bytes = the bytes of it the kernel backs with huge pages now (-1 if
 * /proc/self/smaps cannot be read). Returns 0, or 2 for null arguments or a
 * pointer orth_gb300_host_alloc did not return.
 */
int orth_gb300_host_alloc(size_t bytes, void **ptr);
int orth_gb300_host_free(void *ptr);
int orth_gb300_host_buffer_info(const void *ptr, int *kind, long long *huge_bytes);

/*
 * Row-sharded runs: one rank per GPU, each holding a contiguous block of rows
 * of X, as the reference's MPI ranks do (SRC/orth.c:69-76 partitions m rows;
 * every MPI_Allreduce sums the ranks' partial Gram blocks). The partition is the
 * reference's rule applied to chunks of ORTH_GB300_SHARD_ROWS rows:
 * orth_gb300_shard_rows gives this rank's first row and row count (host
 * arithmetic, no GPU; 2 if some rank would get no chunk). Each rank then calls
 * orth_gb300_run_sharded with its rows (dXsub: msub x n, ldX >= msub, device
 * memory, overwritten with its rows of Q) and a full n x n dR (device memory,
 * written on every rank). Only FP64 (the reference's arithmetic).
 *
 * Instead of an allreduce, each synchronization gathers every rank's per-chunk
 * partial Gram sums and adds them in global chunk order on every rank, and the
 * TSQR gathers its leaf tiles' R factors and runs the upper tree on every rank.
 * So Q and R do not depend on the number of ranks: they are bit-identical to a
 * one-rank call of orth_gb300_run_sharded on all of X.
 *
 * comm->allgather(ctx, send, recv, count, stream) must copy `count` doubles from
 * `send` on every rank into recv[r * count ...] for r = 0 .. size-1 (device
 * pointers on this rank's GPU), ordered after the work enqueued on `stream`
 * before the call and before the work enqueued after it returns: e.g.
 * ncclAllGather on that stream, or a stream synchronize plus a host-staged
 * MPI_Allgather. It returns 0 on success. The callback is called from the
 * calling thread only. Return codes as orth_gb300_run_dev, plus 2 for an
 * invalid communicator or partition. Synchronizes the stream before returning.
 */
#define ORTH_GB300_SHARD_ROWS 8192
typedef int (*orth_gb300_allgather_fn)(void *ctx, const double *send, double *recv, long long count,
                                       void *stream);
typedef struct orth_gb300_comm {
    int rank, size;
    orth_gb300_allgather_fn allgather;
    void *ctx;
} orth_gb300_comm;
int orth_gb300_shard_rows(long long m, int size, int rank, long long *row0, long long *msub);
int orth_gb300_run_sharded(int variant, long long m, int n, int s, double *dXsub, long long ldX,
                           double *dR, int ldR, void *stream, const orth_gb300_comm *comm,
                           orth_gb300_status *status);

/*
 * IntraOrtho of the panels the reference factors with Trilinos TSQR (block 1 of
 * every variant, SRC/orth.c:105-107 and its counterparts; each step's panels in
 * bcgsi2, :520-523 and :532-535, and in bcgsi2P2s, :612-614 and :649-652):
 *   ORTH_GB300_INTRA_TSQR     the hand-written TSQR tree (default, the reference's choice)
 *   ORTH_GB300_INTRA_CHOLQR2  CholeskyQR2: twice G = V^T V (one deterministic
 *                             reduction each), T = chol(G), V = V T^{-1}; R = R2 R1.
 *                             Cheaper (two tall passes), but its Cholesky breaks down
 *                             for panels with condition number beyond about 1e8;
 *                             a breakdown is reported like a Pythagorean one (status
 *                             breakdown_step = the block step).
 * Applies to the orth.h entry points and orth_gb300_run_dev, in every precision
 * (the panel factorization runs in FP64); batched plans and the allocation-free
 * entry point always use TSQR. The environment variable ORTH_GB300_INTRA = tsqr |
 * cholqr2 sets it at first use. Returns 0, or 2 for an unknown mode.
 */
#define ORTH_GB300_INTRA_TSQR 0
#define ORTH_GB300_INTRA_CHOLQR2 1
int orth_gb300_set_intra_ortho(int mode);

/*
 * Diagnostic of the split-precision kernels: the last nonzero error word, i.e. the
 * code of a bounded wait that ran out (for the operand-ring waits, code + 100 *
 * ring slot), or 0 if none has.
 */
int orth_gb300_last_split_error(void);

/* 1 if the split-precision mode handles (m, n, s) (s <= 64), else 0. */
int orth_gb300_split_supported(int m, int n, int s);

/*
 * One "synchronization" on its own: C (na x nb, ldc) = X[:, 0:na]^T X[:, b0:b0+nb]
 * for device X (m rows, ldX), in FP64 or split precision, deterministic. The
 * reference computes it as dgemm('T','N') followed by MPI_Allreduce (for example
 * SRC/orth.c:182-188). Waits for the stream. Return codes as orth_gb300_run_dev.
 */
int orth_gb300_gram_dev(int m, int na, int b0, int nb, const double *dX, long long ldX,
                        double *dC, int ldc, int precision, void *stream);

/*
 * Accuracy of a finished QR, on the device: the GPU form of the reference's
 * test_orth_accuracy (SRC/util.c:36-75, which prints ||Q^T Q - I||_F and
 * ||Q R - X||_F). dX: the original m x n matrix (ldX); dQ: the computed Q (ldQ);
 * dR: the computed R (n x n, ldR; read as upper triangular).
 *   out[0] = ||Q^T Q - I||_F, out[1] = ||Q R - X||_F, out[2] = ||X||_F.
 * gram_precision selects how Q^T Q is formed: ORTH_GB300_FP64 (FP64 Gram kernel)
 * or ORTH_GB300_SPLIT_BF16 (tensor-core digit Gram with exact accumulation; needs
 * orth_gb300_split_supported(m, n, 16)). dE, if not NULL, receives the symmetric
 * n x n error Q^T Q - I (lde >= n) for a 2-norm. Sums of squares are accumulated
 * in double-double in a fixed order. Synchronizes the stream.
 * Returns 0, 2 (invalid arguments), 3 (CUDA failure) or 4 (precision not
 * available for this shape).
 */
int orth_gb300_accuracy_dev(int m, int n, const double *dX, long long ldX, const double *dQ, long long ldQ,
                            const double *dR, int ldR, int gram_precision, double *dE, int lde, void *stream,
                            double out[3]);

/*
 * The split form's digit planes of a matrix, for tests of the slicing: each column
 * c of X (m x n, ldX >= m) is scaled by 2^-e_c, e_c the exponent with max |X[:, c]|
 * < 2^e_c (Inf and NaN ignored; 0 for a zero column), rounded to the fixed point
 * V = round(x * 2^(8 planes - 1 - e_c)) (half away from zero) and split into
 * `planes` (6 or 7) balanced base-256 digits d_0 (most significant) .. in
 * [-128, 128], stored as BF16 bits. dDigits (planes * ceil(m/64) * 64 * n
 * unsigned shorts) receives them in the store's layout: digit i of X[r, c] at
 * ((i * ceil(m/64) + r/64) * n + c) * 64 + r % 64, rows past m as digits of zero;
 * dExp[n] receives e_c. Synchronizes the stream. Returns 0, 2 (invalid arguments,
 * or n > 65535) or 3 (CUDA failure).
 */
int orth_gb300_split_slice_dev(long long m, int n, const double *dX, long long ldX, int planes,
                               unsigned short *dDigits, int *dExp, void *stream);

/*
 * Rows per chunk of the FP64 Gram's fixed-order reduction (0 = the default policy:
 * the most chunks whose 16-column strip CTAs all fit on the SMs in one wave, at
 * least 256 rows each). Results depend on the chunking only through the order
 * of the final sum; a batched plan with the same chunk rows reproduces the
 * single-matrix results bit for bit.
 */
void orth_gb300_set_gram_chunk_rows(long long rows);

/*
 * Batched form: many independent BCGSI+P-1S QRs (the reference's bcgsi2P1s on each
 * matrix) run as one captured CUDA graph, one launch per stage for all matrices.
 * Matrix b: dX[b] (m[b] x n[b], ldX[b] >= m[b], overwritten with Q), dR[b]
 * (n[b] x n[b], ldR[b]; upper block triangle written), block size s[b] <= 16,
 * n[b] >= 2 s[b], m[b] >= n[b]. Arrays are host arrays of count entries (ldX/ldR
 * may be NULL: tight). precision ORTH_GB300_FP64: variant ORTH_GB300_BCGSI2P1S,
 * s[b] <= 16. flags: ORTH_GB300_BATCH_TUNE times the Gram's panel width and chunk
 * rows per block size on the batch itself (reads X, writes only the plan's
 * scratch).
 * precision ORTH_GB300_SPLIT_BF16 / _FAST:
 *   - ORTH_GB300_BCGSI2P1S with every s[b] <= 16 (the default form): staged
 *     graphs. The matrices are taken in order into waves whose digit stores
 *     (14 bytes per element) and scratch fit in 85 % of the free device memory at
 *     creation (or in ORTH_GB300_SPLIT_WAVE_BYTES bytes, when that environment
 *     variable is set); in a wave every stage of the split driver (slicing, the
 *     tensor-core Gram and its reduction, the small FP64 operations, the factor,
 *     its digits, the fused update; the TSQR of block 1) is one launch over all
 *     its matrices, and each wave is one captured CUDA graph; a run replays the
 *     wave graphs in order on `stream`. Each matrix's Q and R are bit-identical to
 *     orth_gb300_run_dev's in the same precision.
 *   - any variant, s[b] <= 64 (and the flags ORTH_GB300_BATCH_STREAMS or
 *     ORTH_GB300_BATCH_ONE_STREAM): each run spreads the matrices over up to 16
 *     scratch slots (as many as fit in half of the free device memory; longest
 *     first to the least loaded slot), each on its own stream forked from and
 *     joined back into `stream`, and runs them through the single-matrix
 *     tensor-core driver (no graph). The slots are the library's own scratch:
 *     order any later library call after the run (same stream, or a synchronize).
 *   Breakdowns and split-kernel timeouts are collected per matrix on the device.
 * The plan owns its device workspace; runs must not overlap.
 * Returns 0, 2 (invalid arguments), 3 (CUDA failure), 4 (variant/precision not
 * available in batched form).
 */
typedef struct orth_gb300_batch orth_gb300_batch;
#define ORTH_GB300_BATCH_TUNE 1
/* Split-precision batches: use one stream and one scratch slot (less device memory). */
#define ORTH_GB300_BATCH_ONE_STREAM 2
/* Split-precision batches: the per-matrix driver on concurrent streams instead of staged graphs. */
#define ORTH_GB300_BATCH_STREAMS 4
int orth_gb300_batch_create(orth_gb300_batch **plan, int variant, int count, const int *m, const int *n,
                            const int *s, double *const *dX, const long long *ldX, double *const *dR,
                            const int *ldR, int precision, int flags, void *stream);
/* Enqueue one run of the whole batch (a graph launch) on stream. */
int orth_gb300_batch_run(orth_gb300_batch *plan, void *stream);
/* Per-matrix Cholesky breakdown (step, info; 0 if none) of the last run; waits for the device. */
int orth_gb300_batch_status(orth_gb300_batch *plan, int *breakdown_step, int *breakdown_info, int *nbroken);
/* Kernel launches per run, device bytes held, graph nodes, and the tuned
 * (panel width, chunk rows) for s <= 4, <= 8, <= 16 (tuned: 6 ints). */
int orth_gb300_batch_info(const orth_gb300_batch *plan, long long *launches_per_run, long long *workspace_bytes,
                          int *graph_nodes, int *tuned);
void orth_gb300_batch_destroy(orth_gb300_batch *plan);
/* The schedule without a GPU: stages, launches per run and device bytes a plan
 * for these shapes would hold. */
/*
 * The staged split-precision plan of a batch, without a GPU: how many waves a
 * wave budget of budget_bytes gives, the kernel launches of one run, and the
 * bytes of the largest wave's device buffer. 0, 2 (invalid shapes) or 4 (s > 16).
 */
int orth_gb300_split_batch_dry_run(int count, const int *m, const int *n, const int *s, long long budget_bytes,
                                   int *waves, long long *launches_per_run, long long *wave_bytes);

int orth_gb300_batch_dry_run(int count, const int *m, const int *n, const int *s, long long *stages,
                             long long *launches_per_run, long long *workspace_bytes);
/* The schedule of a split-precision batch without a GPU: returns the number of
 * scratch slots S a run would use when free_bytes of device memory are free
 * (free_bytes < 0: no memory limit; max_slots >= 1 caps S), and fills slot_of[b]
 * (the slot of matrix b) and order[b] (the b-th matrix enqueued: longest job
 * m n^2 first, each to the least loaded slot). Either array may be NULL. 0 for
 * invalid arguments. */
int orth_gb300_split_batch_plan(int count, const int *m, const int *n, const int *s, long long free_bytes,
                                int max_slots, int *slot_of, int *order);

/*
 * Diagnostic: fill every SM's shared memory with the 64-bit pattern `bits` (e.g. a
 * NaN), on `stream`. A later kernel that reads shared memory it did not write
 * then reads that pattern, so such reads become visible in results. 0 or 3.
 */
int orth_gb300_poison_shared_memory(unsigned long long bits, void *stream);

/*
 * Diagnostic of the failure path: one GPU thread waits, with the bounded wait of
 * the tensor-core kernels (2 s), on an mbarrier that nothing completes. The wait
 * gives up, records `code` (nonzero) and sets its abort flag; the kernel returns.
 * out[0] receives the recorded code (-1 if the wait had succeeded), out[1] the
 * abort flag. Synchronizes the stream. 0, 2 (invalid arguments) or 3.
 */
int orth_gb300_timeout_probe(int code, void *stream, int out[2]);

/* Status of the last run through the orth.h entry points on this thread. */
void orth_gb300_last_status(orth_gb300_status *status);

/*
 * Timeline of the last successful orth.h host-buffer run on this thread, in ms:
 * out[0] all of X on the device, out[1] the QR's kernels done, out[2] last Q
 * chunk back on the host, each from the run's first device operation; out[3] the
 * call's wall time. Zeros before the first such run.
 */
void orth_gb300_last_host_timing(double out[4]);

/*
 * Number of device-wide reductions ("synchronizations") a call performs, from
 * the variant's structure: each replaces one MPI_Allreduce of the reference
 * (SRC/orth.c:113,132 then :187 or :196 per step for bcgsi2P1s; :277,286 then
 * :332 or :341 for bcgsi21s; :423,437 per step for bcgspipi2; :514,526 for
 * bcgsi2; :607,619 then :663 or :672 for bcgsi2P2s).
 */
int orth_gb300_sync_count(int variant, int n, int s);

/*
 * Number of device-wide reductions the last run on this thread actually
 * launched: the fixed-order reduction kernel that replaces each MPI_Allreduce,
 * counted at its launch site. Equals orth_gb300_sync_count for a run that
 * completed.
 */
long long orth_gb300_last_reduction_count(void);

/* Number of kernel launches the last run enqueued (for launch accounting). */
long long orth_gb300_last_launch_count(void);

/*
 * Per-kernel-class timing. orth_gb300_profile(1) resets the accumulators and
 * records a CUDA event pair on the launching stream around every kernel group
 * of later runs; orth_gb300_profile_read waits for them and returns, per class, the
 * summed milliseconds, kernel launches, and algorithmic flops and bytes.
 * Algorithmic bytes are FP64-equivalent in every precision: 8 bytes per element
 * of each operand column the product reads once and each column it writes.
 * Classes: 0 tall Gram + reduction, 1 tall update, 2 small s x s kernels,
 * 3 TSQR, 4 digit slicing (split modes). Arrays have
 * orth_gb300_profile_classes() entries; any may be NULL. Returns 0 or a
 * cudaError_t.
 */
void orth_gb300_profile(int on);
int orth_gb300_profile_classes(void);
int orth_gb300_profile_read(double *ms, long long *launches, double *flops, double *bytes);

/*
 * Per class, the bytes the kernels as built move at least, accumulated like
 * orth_gb300_profile_read's (call it after that): equal to the algorithmic
 * bytes for the FP64 form; for the split forms the operands' BF16 digit planes
 * (2 bytes x digits per element) plus the FP64 columns written. calls[c]: the
 * number of primitive calls (one Gram, one update, ...) timed in class c.
 * Either array may be NULL. Returns 0.
 */
int orth_gb300_profile_traffic(double *bytes, long long *calls);

/* Measure the FP64 pipe's throughput (TFLOP/s) with a DFMA loop; 0 or a cudaError_t. */
int orth_gb300_fp64_peak_probe(double *tflops);

/* Pre-size the cached device workspace for (m, n, s); 0 on success. */
int orth_gb300_reserve(int m, int n, int s);

/* Free the cached device workspace and staging buffers. */
void orth_gb300_release(void);

/* Library version string. */
const char *orth_gb300_version(void);

#ifdef __cplusplus
}
#endif

#endif
