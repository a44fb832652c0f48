// Batched form of the FP64 kernels: one launch runs the same stage of many
// independent QRs. Every launch gets an array of per-matrix jobs and the prefix
// sums of their CTA counts; CTA b finds its job by binary search over the prefix
// array (jobs[j] owns CTAs prefix[j] .. prefix[j+1]-1) and then runs the same body
// as the single-matrix kernel, so every matrix gets the single-matrix arithmetic.
#pragma once

#include <cuda_runtime.h>

namespace bcgs {

using i64 = long long;

// Gram partials + their reduction for one matrix: C = X[:, 0:na]^T X[:, b0:b0+nb].
struct GramJob {
    const double* X;
    i64 ld, m;
    int na, b0, nb, nchunks;
    i64 rows_per_chunk;
    double* part;   // nchunks * na * nb doubles
    double* C;
    int ldc;
    int tb;         // B-panel width: 8, 16 or 32 (A-panel height 512 / tb)
    int tilesA, tilesB;
};

// X[:, c0:c0+nc] = (X[:, c0:c0+nc] - X[:, q0:q0+K] S) T^{-1}, nc <= 16.
struct UpdJob {
    double* X;
    i64 ld, m;
    int q0, K, c0, nc;
    const double* S;
    int lds;
    const double* T;
    int ldt;
};

// Small s x s operations of one matrix, run in order by one CTA.
enum SmallKind { kSmallNone = 0, kSmallPyth = 1, kSmallScol = 2, kSmallRblock = 3 };
struct SmallSub {
    int kind;
    int a, b, c, d, step;
    const double *p0, *p1, *p2, *p3;
    int ld0, ld1, ld2, ld3;
    double* out;
    int ldo;
};
constexpr int kMaxSmallSubs = 4;
struct SmallJob {
    SmallSub sub[kMaxSmallSubs];
    int nsub;
    int* status;
    double* R;
    int ldR;
};

// TSQR: tiles of one level (Q in place, R factors to Rst), the root sign fix, and
// the down-sweep multiply of one level.
struct TsqrTileJob {
    double* A;
    i64 lda, rows;
    int nc;
    double* Rst;
    i64 ldr;
};
struct TsqrRootJob {
    double* Q;
    i64 ldq;
    int hq, nc;
    const double* R;
    i64 ldr;
    double* Rout;
    int ldro;
};
struct TsqrApplyJob {
    double* Q;
    i64 ldq, rows;
    int nc, TR;
    const double* P;
    i64 ldp;
};

// Sets the batched tile kernel's shared-memory limit on the current device
// (outside any stream capture).
int tsqr_tile_batched_prepare();

// Launchers (items = prefix[njobs] CTAs).
int gram_batched_panel_rows(int tb);   // A-panel height for a B-panel width
int launch_gram_partial_batched(const GramJob* jobs, const int* prefix, int njobs, int items, cudaStream_t st);
int launch_gram_reduce_batched(const GramJob* jobs, const int* prefix, int njobs, int items, cudaStream_t st);
int launch_update_batched(const UpdJob* jobs, const int* prefix, int njobs, int items, cudaStream_t st);
int launch_small_batched(const SmallJob* jobs, int njobs, cudaStream_t st);
int launch_tsqr_tile_batched(const TsqrTileJob* jobs, const int* prefix, int njobs, int items, int ncmax,
                             cudaStream_t st);
int launch_tsqr_root_batched(const TsqrRootJob* jobs, int njobs, cudaStream_t st);
int launch_tsqr_apply_batched(const TsqrApplyJob* jobs, const int* prefix, int njobs, int items, int ncmax,
                              cudaStream_t st);

// Job of CTA `item` (prefix[j] <= item < prefix[j + 1]).
__device__ __forceinline__ int batched_job_of(const int* __restrict__ prefix, int njobs, int item) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

}  // namespace bcgs
