// IntraOrtho: explicit TSQR of a tall m x nc panel in FP64 (nc <= 64).
//
// Replaces the reference's Trilinos TSQR::Tsqr::factorExplicit (SRC/orth.c:14-46,
// call sites :107,:271,:413,:505,:522,:534,:601,:613,:651). Trilinos is not part of
// the reference, so the algorithm here is the published TSQR reduction tree:
//
//   level 0: the panel is cut into tiles of TR rows; one CTA of 1-4 warps per
//            tile computes a Householder QR of its tile in shared memory (warp
//            butterfly sums; the warps share out the columns each reflector is
//            applied to), writes the explicit tile Q in place and its nc x nc R
//            into the next level's stack.
//   level l: the stacked R factors (a (tiles * nc) x nc matrix) are cut into tiles
//            of TR rows again and factored the same way, until one tile remains.
//   root   : R is sign-normalized (diag(R) >= 0, the column signs moved into Q).
//   down   : each level's tile Q is multiplied by its nc x nc block of the level
//            above, from the root down to the panel, giving the explicit Q.
//
// Every reduction is in a fixed order (warp butterfly sums, a fixed tree), so
// results are bit-identical run to run.
#include "batched.h"
#include "common.cuh"
#include "kernels.h"

namespace bcgs {

// Tile rows and warps per tile of the single-panel tile kernel by template width.
// All tiles hold 256 rows (BCGS_TSQR_TR64 for nc > 32). A level of the tree
// divides the row count by TR / nc, so taller tiles mean fewer levels and fewer
// flops, at the price of fewer tiles resident per SM. The reflector application
// is split over W warps by groups of columns. Measured on GB300 at m = 2^23,
// n = 512 (TSQR of block 1 per BCGSI+P-1S QR), 256-row tiles (one per SM at
// nc = 64): nc = 64 with 4 warps 431 ms, 8 warps 353 ms, 16 warps 346 ms; nc = 32
// with 2 warps 69.6 ms, 4 warps 64.2 ms, 8 warps 71.4 ms; nc = 16 with one warp
// 16.4 ms. (With the earlier per-warp reflectors and per-column butterflies,
// 128-row tiles were slower at every warp count: 632 ms with 4 warps at nc = 64.)
#ifndef BCGS_TSQR_TR64
#define BCGS_TSQR_TR64 256
#endif
#ifndef BCGS_TSQR_W64
#define BCGS_TSQR_W64 16
#endif
#ifndef BCGS_TSQR_W32
#define BCGS_TSQR_W32 4
#endif
template <int NC>
constexpr int tsqr_tr() { return NC <= 32 ? 256 : BCGS_TSQR_TR64; }
template <int NC>
constexpr int tsqr_tile_warps() { return NC > 32 ? BCGS_TSQR_W64 : (NC > 16 ? BCGS_TSQR_W32 : 1); }

int tsqr_tile_rows(int nc) { return nc <= 32 ? 256 : BCGS_TSQR_TR64; }

// Shared memory of one tile: the TR x NC tile, column-major (ld TR), its NC
// Householder scalars, and two TR-row slots for tau * v of the reflector being
// applied and the next one.
static size_t tsqr_tile_smem_bytes(int TR, int NC) { return (size_t)(TR * NC + NC + 2 * TR) * sizeof(double); }

// Sum of one value over the warp by an xor butterfly. Lane pairs add the same two
// operands (a + b == b + a), so every lane ends with the same bits.
__device__ __forceinline__ double warp_sum1(double w) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    return w;
}

// One reflector H = I - t v v^T applied to column c: w = sum_r v[r] a[r][c] (lane
// `lane` owns rows lane + 32 i, i < RPL), then a[r][c] -= w (t v[r]) with tv = t v.
// v is zero above the reflector's pivot row, so those rows keep their values.
template <int RPL>
__device__ __forceinline__ void apply1(double* a, int TR, int c, const double* v, const double* tv, int lane) {
    double w = 0.0;
#pragma unroll
    for (int i = 0; i < RPL; ++i) w = fma(v[i], a[c * TR + lane + 32 * i], w);
    w = warp_sum1(w);
#pragma unroll
    for (int i = 0; i < RPL; ++i) {
        double* e = &a[c * TR + lane + 32 * i];
        *e = fma(-w, tv[i], *e);
    }
}

// The same for the four columns c0 .. c0+3. The four sums are reduced together:
// lane bit 4 splits the columns into pairs and bit 3 into singles (each lane adds
// the partner's half it keeps), then bits 2-0 finish one column per group of 8
// lanes by a butterfly; lanes 8g .. 8g+7 end with column g's sum, which is then
// broadcast. Six FP64 additions per lane for four columns instead of twenty, in a
// fixed order.
template <int RPL>
__device__ __forceinline__ void apply4(double* a, int TR, int c0, const double* v, const double* tv, int lane) {
    double w[4];
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        w[g] = 0.0;
#pragma unroll
        for (int i = 0; i < RPL; ++i) w[g] = fma(v[i], a[(c0 + g) * TR + lane + 32 * i], w[g]);
    }
    const bool b4 = (lane & 16) != 0, b3 = (lane & 8) != 0;
    double k0 = b4 ? w[2] : w[0], k1 = b4 ? w[3] : w[1];
    const double s0 = b4 ? w[0] : w[2], s1 = b4 ? w[1] : w[3];
    k0 += __shfl_xor_sync(0xffffffffu, s0, 16);
    k1 += __shfl_xor_sync(0xffffffffu, s1, 16);
    double k = b3 ? k1 : k0;
    k += __shfl_xor_sync(0xffffffffu, b3 ? k0 : k1, 8);
    k += __shfl_xor_sync(0xffffffffu, k, 4);
    k += __shfl_xor_sync(0xffffffffu, k, 2);
    k += __shfl_xor_sync(0xffffffffu, k, 1);
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        const double wg = __shfl_sync(0xffffffffu, k, 8 * g);
#pragma unroll
        for (int i = 0; i < RPL; ++i) {
            double* e = &a[(c0 + g) * TR + lane + 32 * i];
            *e = fma(-wg, tv[i], *e);
        }
    }
}

// Applies (v, tv) to the columns of group q (columns [4q, 4q + 4)) that lie in
// [c_lo, nc): four at once when the whole group does.
template <int RPL>
__device__ __forceinline__ void apply_group(double* a, int TR, int q, int c_lo, int nc, const double* v,
                                            const double* tv, int lane) {
    const int g0 = 4 * q;
    if (g0 >= c_lo && g0 + 4 <= nc) {
        apply4<RPL>(a, TR, g0, v, tv, lane);
        return;
    }
    for (int c = g0 > c_lo ? g0 : c_lo; c < g0 + 4 && c < nc; ++c) apply1<RPL>(a, TR, c, v, tv, lane);
}

template <int W>
__device__ __forceinline__ void tile_sync() {
    if (W == 1) __syncwarp(); else __syncthreads();
}

// Householder reflector of column c by the conventions of LAPACK's dlarfg
// (beta = -sign(alpha) sqrt(alpha^2 + ||x||^2), tau = (beta - alpha)/beta,
// v = x / (alpha - beta)), computed by one warp from the column in shared memory
// and stored back in place: v below the diagonal, beta on it, tau in tau[c].
template <int RPL>
__device__ __forceinline__ void make_reflector(double* a, double* tau, double* tvb, int TR, int c, int lane) {
    __syncwarp();   // the column's rows were just written by this warp's lanes
    double x[RPL];
    double p = 0.0;
#pragma unroll
    for (int i = 0; i < RPL; ++i) {
        const int r = lane + 32 * i;
        x[i] = a[c * TR + r];
        if (r > c) p = fma(x[i], x[i], p);
    }
    p = warp_sum1(p);
    const double alpha = a[c * TR + c];
    double t = 0.0, beta = alpha, scal = 0.0;
    if (p > 0.0) {
        beta = -copysign(sqrt(alpha * alpha + p), alpha);
        t = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
    }
    __syncwarp();
    double* tv = tvb + (c & 1) * TR;
#pragma unroll
    for (int i = 0; i < RPL; ++i) {
        const int r = lane + 32 * i;
        const double vr = x[i] * scal;
        if (r > c) a[c * TR + r] = vr;
        else if (r == c) a[c * TR + r] = beta;
        tv[r] = r > c ? t * vr : (r == c ? t : 0.0);
    }
    if (lane == 0) tau[c] = t;
}

// tau_c * v_c of the reflector stored in column c, into slot c & 1 (one warp).
template <int RPL>
__device__ __forceinline__ void publish_tv(const double* a, const double* tau, double* tvb, int TR, int c,
                                           int lane) {
    const double t = tau[c];
    double* tv = tvb + (c & 1) * TR;
#pragma unroll
    for (int i = 0; i < RPL; ++i) {
        const int r = lane + 32 * i;
        tv[r] = r > c ? t * a[c * TR + r] : (r == c ? t : 0.0);
    }
}

// Reflector j (stored in column j) into registers: v (1 on the diagonal, zero
// above) and tv = tau_j v from its published slot.
template <int RPL>
__device__ __forceinline__ double load_reflector(const double* a, const double* tau, const double* tvb, int TR,
                                                 int j, int lane, double* v, double* tv) {
    const double t = tau[j];
    const double* tj = tvb + (j & 1) * TR;
#pragma unroll
    for (int i = 0; i < RPL; ++i) {
        const int r = lane + 32 * i;
        v[i] = r > j ? a[j * TR + r] : (r == j ? 1.0 : 0.0);
        tv[i] = tj[r];
    }
    return t;
}

// W warps per tile, the tile in shared memory (lane L owns rows L, L+32, ...).
// A: rows x nc (lda); tile `tile` covers rows [tile*TR, min(rows, (tile+1)*TR)).
// Householder QR by the conventions of LAPACK's dgeqr2/dlarfg, then the tile's R
// (upper, lower part zero) to Rst rows [tile*nc, (tile+1)*nc) (ld ldr), then the
// explicit tile Q formed in place in dorg2r's order (backward over the reflectors)
// and written to Q (ldq; may alias A). Tiles shorter than nc rows are padded with
// zero rows; padded rows of Q are not written. smem holds
// tsqr_tile_smem_bytes(TR, NC).
//
// The columns are dealt out in groups of four, group q to warp q mod W, and every
// column is only ever updated by its group's warp. Each reflector is formed once,
// by the warp owning its column, and published in shared memory: while applying
// reflector j, the owner of column j+1 updates that column first and forms
// reflector j+1 from it before its other columns (look-ahead), so one barrier per
// reflector separates the steps. Every sum has a fixed order, so the result is
// bit-identical run to run (for a given W).
template <int NC, int W>
__device__ void tsqr_tile_body(const double* A, i64 lda, i64 rows, int nc, double* Q, i64 ldq,
                               double* __restrict__ Rst, i64 ldr, i64 tile, double* smem) {
    constexpr int TR = tsqr_tr<NC>();
    constexpr int RPL = TR / 32;
    double* a = smem;              // a[c * TR + r]
    double* tau = smem + TR * NC;
    double* tvb = tau + NC;        // tau * v of reflectors j and j + 1 (slots j & 1)
    const int lane = threadIdx.x & 31;
    const int warp = W == 1 ? 0 : (int)(threadIdx.x >> 5);
    const int ngroups = (nc + 3) / 4;
    const i64 row0 = tile * TR;
    const i64 h = min((i64)TR, rows - row0);
    tile_sync<W>();
    for (int c = warp; c < nc; c += W)
#pragma unroll
        for (int i = 0; i < RPL; ++i) {
            const int r = lane + 32 * i;
            a[c * TR + r] = (r < h) ? A[row0 + r + (i64)c * lda] : 0.0;
        }
    tile_sync<W>();
    if (warp == 0) make_reflector<RPL>(a, tau, tvb, TR, 0, lane);   // group 0 belongs to warp 0
    tile_sync<W>();

    double v[RPL], tv[RPL];
    for (int j = 0; j < nc; ++j) {
        const double t = load_reflector<RPL>(a, tau, tvb, TR, j, lane, v, tv);
        const int jn = j + 1;
        if (jn < nc) {
            const int qn = jn >> 2;                 // group of column j + 1
            int q0 = qn + ((warp - qn) % W + W) % W; // this warp's first group at or after qn
            if (q0 == qn) {
                if (t != 0.0) apply_group<RPL>(a, TR, qn, jn, nc, v, tv, lane);
                make_reflector<RPL>(a, tau, tvb, TR, jn, lane);
                q0 += W;
            }
            if (t != 0.0)
                for (int q = q0; q < ngroups; q += W) apply_group<RPL>(a, TR, q, jn, nc, v, tv, lane);
        }
        tile_sync<W>();
    }
    // R to the stack (upper, lower zero).
    for (int e = threadIdx.x; e < nc * nc; e += 32 * W) {
        const int i = e % nc, c = e / nc;
        Rst[tile * nc + i + (i64)c * ldr] = (i <= c) ? a[c * TR + i] : 0.0;
    }
    tile_sync<W>();
    // Explicit Q in place (dorg2r): for j = nc-1 .. 0, apply H_j to columns j+1..
    // and set column j to (I - tau v v^T) e_j (its owner, after the barrier that
    // ends every warp's reading of reflector j). tau * v of reflector j - 1 is
    // published during step j by the owner of column j - 1.
    if (((nc - 1) >> 2) % W == warp) publish_tv<RPL>(a, tau, tvb, TR, nc - 1, lane);
    tile_sync<W>();
    for (int j = nc - 1; j >= 0; --j) {
        const double t = load_reflector<RPL>(a, tau, tvb, TR, j, lane, v, tv);
        if (j >= 1 && ((j - 1) >> 2) % W == warp) publish_tv<RPL>(a, tau, tvb, TR, j - 1, lane);
        if (t != 0.0 && j + 1 < nc) {
            const int qn = (j + 1) >> 2;
            for (int q = qn + ((warp - qn) % W + W) % W; q < ngroups; q += W)
                apply_group<RPL>(a, TR, q, j + 1, nc, v, tv, lane);
        }
        tile_sync<W>();
        if ((j >> 2) % W == warp) {
#pragma unroll
            for (int i = 0; i < RPL; ++i) {
                const int r = lane + 32 * i;
                a[j * TR + r] = (r > j) ? -tv[i] : (r == j ? 1.0 - t : 0.0);
            }
        }
    }
    tile_sync<W>();
    for (int c = warp; c < nc; c += W)
#pragma unroll
        for (int i = 0; i < RPL; ++i) {
            const int r = lane + 32 * i;
            if (r < h) Q[row0 + r + (i64)c * ldq] = a[c * TR + r];
        }
    tile_sync<W>();
}

template <int NC>
__global__ void __launch_bounds__(32 * tsqr_tile_warps<NC>())
tsqr_tile_kernel(const double* A, i64 lda, i64 rows, int nc, double* Q, i64 ldq,
                 double* __restrict__ Rst, i64 ldr) {
    extern __shared__ double smem[];
    tsqr_tile_body<NC, tsqr_tile_warps<NC>()>(A, lda, rows, nc, Q, ldq, Rst, ldr, blockIdx.x, smem);
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
    // The whole NC x NC tile: the product below runs over NC terms, and entries
    // past nc must be zeros, not whatever an earlier CTA left in shared memory.
    for (int e = threadIdx.x; e < NC * NC; e += blockDim.x) {
        const int i = e % NC, c = e / NC;
        p[e] = (i < nc && c < nc) ? P[t * nc + i + (i64)c * ldp] : 0.0;
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

// The tree from a given level on: level 0 here is (A0, rows0, ld0), factored in
// place; each level's tile R factors are stacked into the next level (in ws),
// until one tile remains (the root). Then the root's signs are fixed, R is
// written to (R, ldR), and the down-sweep brings the explicit Q back to level 0.
template <int NC>
static int tsqr_levels(double* A0, i64 ld0, i64 rows0, int nc, double* R, int ldR, double* ws, cudaStream_t st) {
    const int TR = tsqr_tile_rows(nc);
    const size_t smem = tsqr_tile_smem_bytes(TR, NC);
    const int attr_rc = smem_attr((const void*)tsqr_tile_kernel<NC>, (int)smem);
    if (attr_rc) return attr_rc;
    constexpr int kMaxLevels = 48;   // each level divides the rows by TR / nc >= 2: 2^k rows need at most k levels
    double* lvl_ptr[kMaxLevels];
    i64 lvl_rows[kMaxLevels], lvl_ld[kMaxLevels];
    lvl_ptr[0] = A0;
    lvl_rows[0] = rows0;
    lvl_ld[0] = ld0;
    int L = 0;
    double* cursor = ws;
    while (lvl_rows[L] > TR) {
        if (L + 1 >= kMaxLevels) return (int)cudaErrorInvalidValue;
        const i64 tiles = ceil_div(lvl_rows[L], TR);
        double* next = cursor;
        cursor += tiles * nc * nc;
        tsqr_tile_kernel<NC><<<(unsigned)tiles, 32 * tsqr_tile_warps<NC>(), smem, st>>>(
            lvl_ptr[L], lvl_ld[L], lvl_rows[L], nc, lvl_ptr[L], lvl_ld[L], next, tiles * nc);
        g_launch_count += 1;
        ++L;
        lvl_ptr[L] = next;
        lvl_rows[L] = tiles * nc;
        lvl_ld[L] = tiles * nc;
    }
    // Root: one tile; its R goes to a small slot after the stacks.
    double* rroot = cursor;
    tsqr_tile_kernel<NC><<<1, 32 * tsqr_tile_warps<NC>(), smem, st>>>(lvl_ptr[L], lvl_ld[L], lvl_rows[L], nc, lvl_ptr[L],
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

template <int NC>
static int tsqr_run(double* X, i64 ld, i64 m, int c0, int nc, double* R, int ldR, double* ws,
                    cudaStream_t st) {
    return tsqr_levels<NC>(X + (i64)c0 * ld, ld, m, nc, R, ldR, ws, st);
}

// Row-sharded TSQR: this rank's rows are the TR-row tiles [t0, t0 + nt) of a
// panel of T tiles. The leaf level runs on the local tiles, writing their R
// factors to `mine` (maxt * nc rows, ld maxt * nc); gather(mine, all) places every
// rank's block in rank order; the blocks are assembled into the global level-1
// stack (T * nc rows, as the one-rank tree has it), whose tree every rank runs;
// the down-sweep of the local tiles then uses this rank's rows of level 1's Q.
// With tiles aligned across ranks, every launch sees the data the one-rank TSQR
// sees, so Q and R are bit-identical to it.
template <int NC>
static int tsqr_sharded_run(double* X, i64 ld, i64 m_local, int c0, int nc, double* R, int ldR, double* ws,
                            const TsqrShard& sh, cudaStream_t st) {
    const int TR = tsqr_tile_rows(nc);
    const size_t smem = tsqr_tile_smem_bytes(TR, NC);
    const int attr_rc = smem_attr((const void*)tsqr_tile_kernel<NC>, (int)smem);
    if (attr_rc) return attr_rc;
    if (sh.T <= 1) return tsqr_run<NC>(X, ld, m_local, c0, nc, R, ldR, ws, st);   // one tile: one rank holds it
    double* panel = X + (i64)c0 * ld;
    const i64 nt = ceil_div(m_local, TR);
    const i64 ldm = sh.maxt * nc;
    if (nt > 0) {
        tsqr_tile_kernel<NC><<<(unsigned)nt, 32 * tsqr_tile_warps<NC>(), smem, st>>>(panel, ld, m_local, nc, panel, ld,
                                                                                   sh.mine, ldm);
        g_launch_count += 1;
    }
    int rc = (int)cudaGetLastError();
    if (rc) return rc;
    rc = sh.gather(sh.ctx, sh.mine, sh.all, ldm * nc, st);
    if (rc) return rc;
    double* lvl1 = ws;
    const i64 ld1 = sh.T * nc;
    for (int r = 0; r < sh.size; ++r) {
        if (sh.nt[r] <= 0) continue;
        rc = (int)cudaMemcpy2DAsync(lvl1 + sh.t0[r] * nc, (size_t)ld1 * sizeof(double), sh.all + (i64)r * ldm * nc,
                                    (size_t)ldm * sizeof(double), (size_t)(sh.nt[r] * nc) * sizeof(double), (size_t)nc,
                                    cudaMemcpyDeviceToDevice, st);
        if (rc) return rc;
    }
    rc = tsqr_levels<NC>(lvl1, ld1, ld1, nc, R, ldR, ws + ld1 * nc, st);
    if (rc) return rc;
    if (nt > 0) {
        tsqr_apply_kernel<NC><<<(unsigned)ceil_div(m_local, 128), 128, 0, st>>>(panel, ld, m_local, nc, TR,
                                                                                 lvl1 + sh.t0[sh.rank] * nc, ld1);
        g_launch_count += 1;
    }
    return (int)cudaGetLastError();
}

int launch_tsqr_sharded(double* X, i64 ld, i64 m_local, int c0, int nc, double* R, int ldR, double* ws,
                        const TsqrShard& sh, cudaStream_t st) {
    if (nc <= 0) return 0;
    if (nc <= 8) return tsqr_sharded_run<8>(X, ld, m_local, c0, nc, R, ldR, ws, sh, st);
    if (nc <= 16) return tsqr_sharded_run<16>(X, ld, m_local, c0, nc, R, ldR, ws, sh, st);
    if (nc <= 32) return tsqr_sharded_run<32>(X, ld, m_local, c0, nc, R, ldR, ws, sh, st);
    if (nc <= 64) return tsqr_sharded_run<64>(X, ld, m_local, c0, nc, R, ldR, ws, sh, st);
    return (int)cudaErrorInvalidValue;
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
__global__ void __launch_bounds__(32)
tsqr_tile_batched(const TsqrTileJob* __restrict__ jobs, const int* __restrict__ prefix, int njobs) {
    extern __shared__ double smem[];
    const int j = batched_job_of(prefix, njobs, blockIdx.x);
    const TsqrTileJob& J = jobs[j];
    const i64 tile = blockIdx.x - prefix[j];
    if (J.nc <= 8)
        tsqr_tile_body<8, 1>(J.A, J.lda, J.rows, J.nc, J.A, J.lda, J.Rst, J.ldr, tile, smem);
    else
        tsqr_tile_body<16, 1>(J.A, J.lda, J.rows, J.nc, J.A, J.lda, J.Rst, J.ldr, tile, smem);
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
    tsqr_tile_batched<<<(unsigned)items, 32, smem, st>>>(jobs, prefix, njobs);
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
