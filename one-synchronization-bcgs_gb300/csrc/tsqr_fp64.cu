// IntraOrtho: explicit TSQR of a tall m x nc panel in FP64 (nc <= 64).
//
// Replaces the reference's Trilinos TSQR::Tsqr::factorExplicit (SRC/orth.c:14-46,
// call sites :107,:271,:413,:505,:522,:534,:601,:613,:651). Trilinos is not part of
// the reference, so the algorithm here is the published TSQR reduction tree:
//
//   level 0: the panel is cut into tiles of TR rows; each CTA computes a
//            Householder QR of its tile in shared memory, writes the explicit tile
//            Q in place and its nc x nc R into the next level's stack.
//   level l: the stacked R factors (a (tiles * nc) x nc matrix) are cut into tiles
//            of TR rows again and factored the same way, until one tile remains.
//   root   : R is sign-normalized (diag(R) >= 0, the column signs moved into Q).
//   down   : each level's tile Q is multiplied by its nc x nc block of the level
//            above, from the root down to the panel, giving the explicit Q.
//
// Every reduction is in a fixed order (block reductions with a fixed warp order,
// a fixed tree), so results are bit-identical run to run.
#include "batched.h"
#include "common.cuh"
#include "kernels.h"

namespace bcgs {

namespace {
constexpr int TQ_MAXW = 8;  // warps in the reduction scratch (TR <= 256)
}

int tsqr_tile_rows(int nc) { return nc <= 32 ? 256 : 128; }

// Block-wide sum of `cnt` per-thread values in v[0..cnt), fixed order. Result in
// out[0..cnt) (shared). Requires blockDim.x == TR (multiple of 32, <= 256).
template <int MAXC>
__device__ __forceinline__ void block_sum_vec(const double* v, int cnt, double* red, double* out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
        if (c >= cnt) break;
        double x = v[c];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
        if (lane == 0) red[warp * MAXC + c] = x;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < cnt; c += blockDim.x) {
        double s = 0.0;
        for (int w = 0; w < nwarps; ++w) s += red[w * MAXC + c];
        out[c] = s;
    }
    __syncthreads();
}

// One CTA per tile. A: rows x nc (lda); tile t covers rows [t*TR, min(rows,(t+1)*TR)).
// Writes the explicit tile Q (same rows) to Q (ldq; may alias A) and the tile R to
// Rst rows [t*nc, (t+1)*nc) (ld ldr), lower part zero. Tiles shorter than nc rows
// are padded with zero rows (their padded Q rows are not written).
// Body shared by the single and batched kernels: tile `tile` of the level matrix;
// smem holds tsqr_tile_smem_doubles(TR, NC) doubles.
template <int NC>
__device__ void tsqr_tile_body(const double* A, i64 lda, i64 rows, int nc, double* Q, i64 ldq,
                               double* __restrict__ Rst, i64 ldr, i64 tile, double* smem) {
    const int TR = blockDim.x;
    const int TRP = TR + 1;
    double* a = smem;                       // TR x NC, column-major, ld TRP
    double* q = a + (size_t)TRP * NC;       // TR x NC
    double* red = q + (size_t)TRP * NC;     // TQ_MAXW x NC
    double* wv = red + TQ_MAXW * NC;        // NC
    double* tau = wv + NC;                  // NC
    __shared__ double s_sc[2];

    const int r = threadIdx.x;
    __syncthreads();
    const i64 row0 = tile * TR;
    const i64 h = min((i64)TR, rows - row0);
    for (int c = 0; c < NC; ++c)
        a[r + c * TRP] = (c < nc && r < h) ? A[row0 + r + (i64)c * lda] : 0.0;
    __syncthreads();

    double part[NC];
    // Householder QR, LAPACK dgeqr2 / dlarfg conventions.
    for (int j = 0; j < nc; ++j) {
        double x = (r > j) ? a[r + j * TRP] : 0.0;
        part[0] = x * x;
        block_sum_vec<1>(part, 1, red, wv);
        const double xnorm2 = wv[0];
        if (r == 0) {
            const double alpha = a[j + j * TRP];
            double t = 0.0, beta = alpha, scal = 0.0;
            if (xnorm2 > 0.0) {
                beta = -copysign(sqrt(alpha * alpha + xnorm2), alpha);
                t = (beta - alpha) / beta;
                scal = 1.0 / (alpha - beta);
            }
            tau[j] = t;
            s_sc[0] = beta;
            s_sc[1] = scal;
        }
        __syncthreads();
        const double beta = s_sc[0], scal = s_sc[1], tj = tau[j];
        double v = 0.0;
        if (r == j) v = 1.0;
        else if (r > j) v = a[r + j * TRP] * scal;
        __syncthreads();
        if (r > j) a[r + j * TRP] = v;
        if (r == j) a[j + j * TRP] = beta;
        // Apply H_j = I - tau v v^T to columns j+1..nc-1.
        const int cnt = nc - j - 1;
        if (cnt > 0 && tj != 0.0) {
#pragma unroll
            for (int c = 0; c < NC; ++c)
                if (c < cnt) part[c] = (r >= j) ? v * a[r + (j + 1 + c) * TRP] : 0.0;
            block_sum_vec<NC>(part, cnt, red, wv);
            if (r >= j) {
                for (int c = 0; c < cnt; ++c) a[r + (j + 1 + c) * TRP] -= tj * wv[c] * v;
            }
        }
        __syncthreads();
    }
    // R to the stack (upper, lower zero).
    for (int e = r; e < nc * nc; e += TR) {
        int i = e % nc, c = e / nc;
        Rst[tile * nc + i + (i64)c * ldr] = (i <= c) ? a[i + c * TRP] : 0.0;
    }
    // Explicit Q = H_0 ... H_{nc-1} [I; 0] (dorg2r), backward accumulation.
    for (int c = 0; c < NC; ++c) q[r + c * TRP] = (c < nc && r == c) ? 1.0 : 0.0;
    __syncthreads();
    for (int j = nc - 1; j >= 0; --j) {
        const double tj = tau[j];
        const double v = (r == j) ? 1.0 : ((r > j) ? a[r + j * TRP] : 0.0);
        if (tj != 0.0) {
#pragma unroll
            for (int c = 0; c < NC; ++c)
                if (c < nc) part[c] = v * q[r + c * TRP];
            block_sum_vec<NC>(part, nc, red, wv);
            if (r >= j)
                for (int c = 0; c < nc; ++c) q[r + c * TRP] -= tj * wv[c] * v;
        }
        __syncthreads();
    }
    if (r < h)
        for (int c = 0; c < nc; ++c) Q[row0 + r + (i64)c * ldq] = q[r + c * TRP];
    __syncthreads();
}

template <int NC>
__global__ void __launch_bounds__(256)
tsqr_tile_kernel(const double* A, i64 lda, i64 rows, int nc, double* Q, i64 ldq,
                 double* __restrict__ Rst, i64 ldr) {
    extern __shared__ double smem[];
    tsqr_tile_body<NC>(A, lda, rows, nc, Q, ldq, Rst, ldr, blockIdx.x, smem);
}

// Root fix-up: make diag(R) >= 0. R (nc x nc, ld ldr) rows with a negative
// diagonal are negated, as are the matching columns of the root Q (hq x nc, ldq).
// The final R is also copied to Rout (ld ldro), lower part zero.
__device__ void tsqr_root_fix_body(double* Q, i64 ldq, int hq, int nc, const double* R, i64 ldr,
                                   double* Rout, int ldro) {
    __shared__ double sgn[64];
    __syncthreads();
    if (threadIdx.x < nc) sgn[threadIdx.x] = (R[threadIdx.x + (i64)threadIdx.x * ldr] < 0.0) ? -1.0 : 1.0;
    __syncthreads();
    for (int e = threadIdx.x; e < nc * nc; e += blockDim.x) {
        int i = e % nc, c = e / nc;
        Rout[i + (i64)c * ldro] = (i <= c) ? sgn[i] * R[i + (i64)c * ldr] : 0.0;
    }
    for (int e = threadIdx.x; e < hq * nc; e += blockDim.x) {
        int i = e % hq, c = e / hq;
        Q[i + (i64)c * ldq] *= sgn[c];
    }
    __syncthreads();
}

__global__ void tsqr_root_fix(double* Q, i64 ldq, int hq, int nc, const double* R, i64 ldr,
                              double* Rout, int ldro) {
    tsqr_root_fix_body(Q, ldq, hq, nc, R, ldr, Rout, ldro);
}

// Down-sweep: for each tile t of TR rows of Q (rows x nc, ldq):
//   Q[tile t] = Q[tile t] * P[t*nc:(t+1)*nc, 0:nc]   (P: ld ldp)
// Body shared by the single and batched kernels: rows [blk*blockDim, ...) of Q.
template <int NC>
__device__ void tsqr_apply_body(double* Q, i64 ldq, i64 rows, int nc, int TR, const double* __restrict__ P,
                                i64 ldp, i64 blk) {
    __shared__ double p[NC * NC];
    __syncthreads();
    const i64 r = blk * blockDim.x + threadIdx.x;
    const i64 t = (blk * blockDim.x) / TR;   // blockDim.x divides TR
    for (int e = threadIdx.x; e < nc * nc; e += blockDim.x) {
        int i = e % nc, c = e / nc;
        p[i + c * NC] = P[t * nc + i + (i64)c * ldp];
    }
    __syncthreads();
    if (r >= rows) return;   // the last statement of the body: no barrier follows
    double x[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) x[c] = (c < nc) ? Q[r + (i64)c * ldq] : 0.0;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        if (c >= nc) break;
        double y = 0.0;
#pragma unroll
        for (int i = 0; i < NC; ++i) y = fma(x[i], p[i + c * NC], y);
        Q[r + (i64)c * ldq] = y;
    }
}

template <int NC>
__global__ void __launch_bounds__(256)
tsqr_apply_kernel(double* Q, i64 ldq, i64 rows, int nc, int TR, const double* __restrict__ P, i64 ldp) {
    tsqr_apply_body<NC>(Q, ldq, rows, nc, TR, P, ldp, blockIdx.x);
}

i64 tsqr_workspace_doubles(i64 m, int nc) {
    const int TR = tsqr_tile_rows(nc);
    i64 total = 0, h = m;
    while (h > TR) {
        i64 tiles = ceil_div(h, TR);
        total += tiles * nc * nc;
        h = tiles * nc;
    }
    return total + 64 * 64;  // + the root tile's R
}

template <int NC>
static int tsqr_run(double* X, i64 ld, i64 m, int c0, int nc, double* R, int ldR, double* ws,
                    cudaStream_t st) {
    const int TR = tsqr_tile_rows(nc);
    const size_t smem = (size_t)(2 * (TR + 1) * NC + TQ_MAXW * NC + 2 * NC) * sizeof(double);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(tsqr_tile_kernel<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        attr_set = true;
    }
    // Level matrices: level 0 is the panel itself; level l >= 1 lives in ws.
    constexpr int kMaxLevels = 16;
    double* lvl_ptr[kMaxLevels];
    i64 lvl_rows[kMaxLevels], lvl_ld[kMaxLevels];
    lvl_ptr[0] = X + (i64)c0 * ld;
    lvl_rows[0] = m;
    lvl_ld[0] = ld;
    int L = 0;
    double* cursor = ws;
    while (lvl_rows[L] > TR) {
        if (L + 1 >= kMaxLevels) return (int)cudaErrorInvalidValue;
        const i64 tiles = ceil_div(lvl_rows[L], TR);
        double* next = cursor;
        cursor += tiles * nc * nc;
        tsqr_tile_kernel<NC><<<(unsigned)tiles, TR, smem, st>>>(
            lvl_ptr[L], lvl_ld[L], lvl_rows[L], nc, lvl_ptr[L], lvl_ld[L], next, tiles * nc);
        g_launch_count += 1;
        ++L;
        lvl_ptr[L] = next;
        lvl_rows[L] = tiles * nc;
        lvl_ld[L] = tiles * nc;
    }
    // Root: one tile; its R goes to a small slot after the stacks.
    double* rroot = cursor;
    tsqr_tile_kernel<NC><<<1, TR, smem, st>>>(lvl_ptr[L], lvl_ld[L], lvl_rows[L], nc, lvl_ptr[L],
                                              lvl_ld[L], rroot, nc);
    tsqr_root_fix<<<1, 256, 0, st>>>(lvl_ptr[L], lvl_ld[L], (int)lvl_rows[L], nc, rroot, nc, R, ldR);
    g_launch_count += 2;
    // Down-sweep.
    for (int l = L - 1; l >= 0; --l) {
        const unsigned blocks = (unsigned)ceil_div(lvl_rows[l], 128);
        tsqr_apply_kernel<NC><<<blocks, 128, 0, st>>>(lvl_ptr[l], lvl_ld[l], lvl_rows[l], nc, TR,
                                                      lvl_ptr[l + 1], lvl_ld[l + 1]);
        g_launch_count += 1;
    }
    return (int)cudaGetLastError();
}

int launch_tsqr(double* X, i64 ld, i64 m, int c0, int nc, double* R, int ldR, double* ws,
                cudaStream_t st) {
    if (nc <= 0) return 0;
    if (nc <= 8) return tsqr_run<8>(X, ld, m, c0, nc, R, ldR, ws, st);
    if (nc <= 16) return tsqr_run<16>(X, ld, m, c0, nc, R, ldR, ws, st);
    if (nc <= 32) return tsqr_run<32>(X, ld, m, c0, nc, R, ldR, ws, st);
    if (nc <= 64) return tsqr_run<64>(X, ld, m, c0, nc, R, ldR, ws, st);
    return (int)cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// Batched forms (batched.h): tiles of one tree level, root sign fixes and one
// down-sweep level over many panels (nc <= 16, TR = 256), with the single-panel
// bodies.
// ---------------------------------------------------------------------------
static size_t tsqr_tile_smem_bytes(int TR, int NC) {
    return (size_t)(2 * (TR + 1) * NC + TQ_MAXW * NC + 2 * NC) * sizeof(double);
}

__global__ void __launch_bounds__(256)
tsqr_tile_batched(const TsqrTileJob* __restrict__ jobs, const int* __restrict__ prefix, int njobs) {
    extern __shared__ double smem[];
    const int j = batched_job_of(prefix, njobs, blockIdx.x);
    const TsqrTileJob& J = jobs[j];
    const i64 tile = blockIdx.x - prefix[j];
    if (J.nc <= 8)
        tsqr_tile_body<8>(J.A, J.lda, J.rows, J.nc, J.A, J.lda, J.Rst, J.ldr, tile, smem);
    else
        tsqr_tile_body<16>(J.A, J.lda, J.rows, J.nc, J.A, J.lda, J.Rst, J.ldr, tile, smem);
}

__global__ void tsqr_root_batched(const TsqrRootJob* __restrict__ jobs) {
    const TsqrRootJob& J = jobs[blockIdx.x];
    tsqr_root_fix_body(J.Q, J.ldq, J.hq, J.nc, J.R, J.ldr, J.Rout, J.ldro);
}

__global__ void __launch_bounds__(128)
tsqr_apply_batched(const TsqrApplyJob* __restrict__ jobs, const int* __restrict__ prefix, int njobs) {
    const int j = batched_job_of(prefix, njobs, blockIdx.x);
    const TsqrApplyJob& J = jobs[j];
    const i64 blk = blockIdx.x - prefix[j];
    if (J.nc <= 8)
        tsqr_apply_body<8>(J.Q, J.ldq, J.rows, J.nc, J.TR, J.P, J.ldp, blk);
    else
        tsqr_apply_body<16>(J.Q, J.ldq, J.rows, J.nc, J.TR, J.P, J.ldp, blk);
}

// Sets the batched tile kernel's shared-memory limit (outside any stream capture).
int tsqr_tile_batched_prepare() {
    return (int)cudaFuncSetAttribute(tsqr_tile_batched, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tsqr_tile_smem_bytes(256, 16));
}

int launch_tsqr_tile_batched(const TsqrTileJob* jobs, const int* prefix, int njobs, int items, int ncmax,
                             cudaStream_t st) {
    if (items <= 0) return 0;
    if (ncmax > 16) return (int)cudaErrorInvalidValue;
    const size_t smem = tsqr_tile_smem_bytes(256, 16);
    tsqr_tile_batched<<<(unsigned)items, 256, smem, st>>>(jobs, prefix, njobs);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

int launch_tsqr_root_batched(const TsqrRootJob* jobs, int njobs, cudaStream_t st) {
    if (njobs <= 0) return 0;
    tsqr_root_batched<<<(unsigned)njobs, 256, 0, st>>>(jobs);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

int launch_tsqr_apply_batched(const TsqrApplyJob* jobs, const int* prefix, int njobs, int items, int ncmax,
                              cudaStream_t st) {
    if (items <= 0) return 0;
    if (ncmax > 16) return (int)cudaErrorInvalidValue;
    tsqr_apply_batched<<<(unsigned)items, 128, 0, st>>>(jobs, prefix, njobs);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

}  // namespace bcgs
