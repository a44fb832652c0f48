// Split-precision tall products on the GB300 tensor cores (tcgen05, BF16 in, FP32
// accumulate), used by the ORTH_GB300_SPLIT_BF16 mode of every variant.
//
// Representation. Each FP64 column c of X is held as KD balanced base-256 digit
// planes with a per-column power-of-two scale 2^e_c (|x| < 2^e_c):
//     x = 2^e_c * sum_{i=1..KD} d_i * 2^{-(8i-1)},   d_i in [-128, 128],
// i.e. 8*KD bits of fixed point (KD = 7: 56 bits, KD = 6: 48 bits). Every digit is an integer of
// at most 8 significant bits, so it is exact in BF16, and a digit product is an
// integer below 2^14, exact in the FP32 accumulator. Products of equal weight
// 2^{2-8(i+j)} are summed in the same TMEM columns: A-plane i is multiplied with the
// concatenation [B_1 .. B_{KD+1-i}] (N = NB*(KD+1-i)) into TMEM column block i-1,
// so block g-2 accumulates every product with i + j = g (products with i + j > KD+1
// are below 2^{-8 KD} and dropped). Block g-2 sums at most g-1 <= 7 products of
// magnitude <= 2^14 per summation step; the accumulators are emptied every 128
// summation steps, so every partial sum stays below 7 * 2^21 < 2^24 and the FP32
// accumulation is exact. Groups g = 2..7 are drained into two exact 64-bit
// integers; group g = 8 (weight 2^-48 relative) is summed in FP32.
//
// One digit store serves both product shapes. It is chunked so that every TMA
// tile is one contiguous block of HBM:
//   column store [plane][64-row chunk][column][64 rows]
// The tall Gram X[:, 0:na]^T X[:, b0:b0+nb] (sum over rows) reads its A and B
// tiles K-major: 64 rows of one column are one 128-byte swizzle row. The update
// [Q | X_k] * B (sum over columns) reads its A tile, 128 rows x 64 columns, from
// two adjacent 64-row chunks of the same store as an MN-major operand: there the
// 128-byte rows run along M. Slicing a column writes 2 bytes per digit per
// element once.
// The update (X_k - Q S) T^{-1} is evaluated as one product
//     [Q | X_k] * [-S T^{-1} ; T^{-1}]
// with the column scales 2^{e_c} folded into the rows of the small right-hand
// factor, so the triangular scaling also runs on the tensor cores.
//
// Kernels are warp-specialized (warp 0: TMA producer, warp 1: MMA issuer + TMEM
// owner, then the epilogue: in the Gram warps 2-9, two threads per TMEM lane; in
// the update warps 2-17, four threads per TMEM lane), with an A-tile ring of
// 16 KB slots, a B ring, and two TMEM accumulators so the epilogue of one window
// overlaps the MMAs of the next. The update is persistent and takes row tiles from
// a per-launch counter; the Gram's M-block CTAs of one row range run side by side
// and share each B tile through L2 (B loaded evict_last, A evict_first). No load
// is multicast. Every wait is bounded; a timeout sets an
// error word and the kernel winds down.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "../../include/orth_gb300.h"
#include "batched.h"
#include "common.cuh"
#include "kernels.h"
#include "split.h"
#include "tc_common.cuh"

namespace bcgs {

namespace {

constexpr int KD_MAX = 7;      // digit planes held by the stores
constexpr int TILE_M = 128;    // MMA M (rows of D = TMEM lanes)
constexpr int KCH = 64;        // K elements per chunk (one 128-byte swizzle row)
constexpr int WIN = 2;         // chunks per accumulation window (128 summation steps)
constexpr int ROW_ALIGN = 256; // Gram row ranges: multiples of 256 rows (whole windows)
constexpr int RA = 8;          // A ring depth (16 KB slots)
constexpr int RB = 2;          // B ring depth
constexpr int A_SLOT = TILE_M * KCH * 2;   // 16 KB
constexpr int NTHREADS = 320;  // Gram: 10 warps: producer, MMA, 8 epilogue
constexpr int NEPI = 256;      // Gram: epilogue threads (two per TMEM lane)
// The update's epilogue drains and assembles every output of every row tile (the
// Gram's only once per CTA), so it has four threads per TMEM lane: 18 warps.
constexpr int UEPW = 4;                     // update: epilogue threads per TMEM lane
constexpr int UNEPI = 128 * UEPW;           // update: epilogue threads
constexpr int UTHREADS = 64 + UNEPI;        // update: producer + MMA warps + epilogue

// ---------------------------------------------------------------------------
// Digit extraction: x -> KD balanced base-256 digits of x * 2^{-e} (|x| < 2^e).
// Integer arithmetic on the FP64 bit pattern only (no FP64 pipe work).
// ---------------------------------------------------------------------------
template <int KD>
__device__ __forceinline__ long long fixed_point_of(double x, int e) {
    // V = round(x * 2^{8 KD - 1 - e}) from the FP64 bit pattern, half away from
    // zero. With |x| < 2^e the mantissa's shift sh = E - 1075 + 8 KD - 1 - e is at
    // most 2, so k = 3 - sh >= 1 and V = (8 M + 2^{k-1}) >> k (exact for sh >= 0,
    // rounded for sh < 0). k is clamped to 63, where the quotient is already 0
    // (8 M < 2^56). Zero, subnormals, Inf and NaN give 0.
    const long long bits = __double_as_longlong(x);
    const int E = (int)((bits >> 52) & 0x7FF);
    if (E == 0 || E == 0x7FF) return 0;
    const unsigned long long M8 = ((unsigned long long)(bits & 0xFFFFFFFFFFFFFLL) | (1ULL << 52)) << 3;
    int k = 3 - (E - 1075 + 8 * KD - 1 - e);
    k = k < 1 ? 1 : (k > 63 ? 63 : k);
    const long long V = (long long)((M8 + (1ULL << (k - 1))) >> k);
    return bits < 0 ? -V : V;
}

// Balanced digits d_0 (most significant) .. d_{KD-1} in [-128, 128] of V. With the
// bias 0x80 added to each of the KD-1 low bytes, byte i of V + bias is d + 128 for
// the low digits and the remaining high part is d_0.
template <int KD>
__device__ __forceinline__ void split_digits(double x, int e, int* d) {
    constexpr unsigned long long kBias = 0x8080808080808080ULL >> (8 * (8 - (KD - 1)));
    const long long Vb = fixed_point_of<KD>(x, e) + (long long)kBias;
#pragma unroll
    for (int i = 1; i < KD; ++i) d[i] = (int)((Vb >> (8 * (KD - 1 - i))) & 255) - 128;
    d[0] = (int)(Vb >> (8 * (KD - 1)));
}

// Exponent e with max < 2^e from the bit pattern of a non-negative max.
__device__ __forceinline__ int scale_exp(unsigned long long maxbits) {
    const int E = (int)((maxbits >> 52) & 0x7FF);
    return E == 0 ? 0 : E - 1022;
}

// BF16 bits of a small integer |d| <= 2^8 (exact: at most 8 significant bits),
// through the FP32 magic constant 1.5 * 2^23 instead of a conversion instruction.
__device__ __forceinline__ unsigned short bf16_bits_of_int(int d) {
    const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
    return (unsigned short)(__float_as_uint(f) >> 16);
}

// Column max |x| (bit patterns of non-negative doubles order like the values):
// rows [4096 rb, 4096 (rb + 1)) of column c into cmax[c].
__device__ __forceinline__ void colmax_body(const double* __restrict__ X, i64 ld, i64 m, int c, int rb,
                                            unsigned long long* __restrict__ cmax) {
    const i64 r0 = (i64)rb * 4096;
    const i64 r1 = min(m, r0 + 4096);
    const double* col = X + (i64)c * ld;
    // 4096 rows over the CTA's threads, all loads of a thread issued before any
    // is used (16 in flight per thread at 256 threads).
    constexpr int kMaxIt = 16;
    unsigned long long v = 0;
    const int step = (int)blockDim.x;
    if (r0 + (i64)step * kMaxIt >= r1) {
        unsigned long long b[kMaxIt];
#pragma unroll
        for (int k = 0; k < kMaxIt; ++k) {
            const i64 r = r0 + threadIdx.x + (i64)k * step;
            b[k] = r < r1 ? ((unsigned long long)__double_as_longlong(col[r]) & 0x7FFFFFFFFFFFFFFFULL) : 0ULL;
        }
#pragma unroll
        for (int k = 0; k < kMaxIt; ++k) {
            const unsigned long long bk = (b[k] >> 52) == 0x7FF ? 0ULL : b[k];   // Inf/NaN do not set the scale
            v = v > bk ? v : bk;
        }
    } else {
        for (i64 r = r0 + threadIdx.x; r < r1; r += step) {
            unsigned long long b = (unsigned long long)__double_as_longlong(col[r]) & 0x7FFFFFFFFFFFFFFFULL;
            if ((b >> 52) == 0x7FF) b = 0;
            v = v > b ? v : b;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = v > w ? v : w;
    }
    __shared__ unsigned long long red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = v > red[w] ? v : red[w];
        v = v > red[0] ? v : red[0];
        atomicMax(cmax + c, v);
    }
}

__global__ void colmax_kernel(const double* __restrict__ X, i64 ld, i64 m, int c0,
                              unsigned long long* __restrict__ cmax) {
    colmax_body(X, ld, m, c0 + (int)blockIdx.y, (int)blockIdx.x, cmax);
}

// BF16 sum of two pairs of BF16 values (exact here: integers of at most 8 bits).
__device__ __forceinline__ uint32_t bf16x2_add(uint32_t a, uint32_t b) {
    uint32_t d;
    asm("add.rn.bf16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}

// The digits of two values of one column (scale exponent e), packed: word i holds
// the BF16 bits of digit i of xa in its low half and of xb in its high half, the
// same bits split_digits + bf16_bits_of_int give. A low digit is byte k of
// V + bias, b = d + 128; with lo = b & 127 and b7 = b & 128, the BF16 words
// 0x4300 | lo (= 128 + lo) and 0xC380 ^ b7 (= -256 + b7) add exactly to
// lo + b7 - 128 = d, two digits per byte permute, two logic operations and one
// BF16x2 add.
template <int KD>
__device__ __forceinline__ void split_digits_pair(double xa, double xb, int e, uint32_t* w) {
    constexpr unsigned long long kBias = 0x8080808080808080ULL >> (8 * (8 - (KD - 1)));
    const unsigned long long va = (unsigned long long)(fixed_point_of<KD>(xa, e) + (long long)kBias);
    const unsigned long long vb = (unsigned long long)(fixed_point_of<KD>(xb, e) + (long long)kBias);
    const uint32_t alo = (uint32_t)va, ahi = (uint32_t)(va >> 32);
    const uint32_t blo = (uint32_t)vb, bhi = (uint32_t)(vb >> 32);
#pragma unroll
    for (int i = 1; i < KD; ++i) {
        const int k = KD - 1 - i;   // byte of V + bias holding digit i
        const uint32_t p = k < 4 ? __byte_perm(alo, blo, (unsigned)(k | ((4 + k) << 8)))
                                 : __byte_perm(ahi, bhi, (unsigned)((k - 4) | (k << 8)));
        w[i] = bf16x2_add((p & 0x007F007Fu) | 0x43004300u, (p & 0x00800080u) ^ 0xC380C380u);
    }
    const int d0a = (int)((long long)va >> (8 * (KD - 1)));
    const int d0b = (int)((long long)vb >> (8 * (KD - 1)));
    w[0] = (uint32_t)bf16_bits_of_int(d0a) | ((uint32_t)bf16_bits_of_int(d0b) << 16);
}

// Slice columns [c0, c0+nc) of X into the digit store. A CTA handles 128 rows x
// 16 columns (grid: row tiles x column groups); thread t makes the digits of rows
// 2u, 2u + 1 (u = t % 64) for 8 of the columns, from one 16-byte load per column
// where the columns start on 16-byte boundaries, two digits per 32-bit word
// (split_digits_pair). The digits are staged in shared memory as [plane][64-row
// half][column][64 rows]. That is the store's own layout: for one plane and one
// 64-row chunk, the 16 columns' runs of 64 rows are one contiguous 2 KB block of
// HBM. A tile of 128 whole rows leaves as 2 KD bulk copies (128 bytes per valid
// column), issued by as many threads; a tile with rows past m is stored
// element-wise.
template <int KD>
__device__ __forceinline__ void slice_body(const double* __restrict__ X, i64 ld, i64 m, int n, int c0, int nc,
                                           const unsigned long long* __restrict__ cmax, int* __restrict__ cexp,
                                           unsigned short* __restrict__ colstore, i64 nrc, int bx, int by) {
    constexpr int CG = 16;                   // columns per CTA
    constexpr int CT = CG / 2;               // columns per thread
    __shared__ __align__(128) uint32_t sw[KD][2][CG][32];
    typedef unsigned short Run[2][CG][64];
    const Run* sdig = reinterpret_cast<const Run*>(&sw[0][0][0][0]);
    const int t = threadIdx.x;
    const int u = t & 63;                    // rows 2u, 2u + 1 of the tile
    const int jt = (t >> 6) * CT;            // the thread's first column of the group
    const int g = by * CG;                   // first column of this group (relative to c0)
    const i64 r0 = (i64)bx * 128;
    const i64 r = r0 + 2 * u;
    if (bx == 0 && t < CG && g + t < nc) cexp[c0 + g + t] = scale_exp(cmax[c0 + g + t]);
    const bool pair = ((reinterpret_cast<uintptr_t>(X) | (uintptr_t)(ld * 8)) & 15) == 0 && r + 1 < m;
    double2 x[CT];
#pragma unroll
    for (int j = 0; j < CT; ++j) {
        const double* p = X + r + (i64)(c0 + g + jt + j) * ld;
        if (g + jt + j >= nc) x[j] = make_double2(0.0, 0.0);
        else if (pair) x[j] = *reinterpret_cast<const double2*>(p);
        else x[j] = make_double2(r < m ? p[0] : 0.0, r + 1 < m ? p[1] : 0.0);
    }
#pragma unroll
    for (int j = 0; j < CT; ++j) {
        const int c = g + jt + j;
        uint32_t w[KD];
        split_digits_pair<KD>(x[j].x, x[j].y, c < nc ? scale_exp(cmax[c0 + c]) : 0, w);
#pragma unroll
        for (int i = 0; i < KD; ++i) sw[i][u >> 5][jt + j][u & 31] = w[i];
    }
    // A tile whose 128 rows all lie below m leaves as bulk copies of its valid
    // columns (ncols x 128 bytes per plane and 64-row half: the store keeps a
    // plane's columns of one chunk contiguous, so a group narrower than 16 columns,
    // as blocks of s = 4 or 8 give, is still one contiguous block).
    const int ncols = nc - g < CG ? nc - g : CG;
    const bool full = r0 + 128 <= m;
    if (full) tc::fence_proxy_async_smem();
    __syncthreads();
    // Element (r, c) of plane i at ((i*nrc + r/64)*n + c)*64 + r%64.
    if (full) {
        if (t < 2 * KD) {
            const int i = t >> 1, h = t & 1;
            unsigned short* dst = colstore + (((i64)i * nrc + r0 / 64 + h) * n + (c0 + g)) * 64;
            tc::bulk_store(dst, &sdig[i][h][0][0], ncols * 64 * 2);
            tc::bulk_commit();
            tc::bulk_wait_read();
        }
        return;
    }
    for (int e = t; e < KD * 2 * CG * 8; e += 128) {
        const int piece = e & 7, rest = e >> 3;     // 16-byte piece of one 64-row run
        const int j = rest % CG, ih = rest / CG;
        const int i = ih >> 1, h = ih & 1;
        if (g + j >= nc) continue;
        const i64 rr = r0 + h * 64 + piece * 8;
        if (rr >= m) continue;
        unsigned short* dst = colstore + (((i64)i * nrc + rr / 64) * n + (c0 + g + j)) * 64 + (rr & 63);
        const unsigned short* src = &sdig[i][h][j][piece * 8];
        for (int q = 0; q < 8; ++q)
            if (rr + q < m) dst[q] = src[q];
    }
}

template <int KD>
__global__ void __launch_bounds__(128, 7)
slice_kernel(const double* __restrict__ X, i64 ld, i64 m, int n, int c0, int nc,
             const unsigned long long* __restrict__ cmax, int* __restrict__ cexp,
             unsigned short* __restrict__ colstore, i64 nrc) {
    slice_body<KD>(X, ld, m, n, c0, nc, cmax, cexp, colstore, nrc, (int)blockIdx.x, (int)blockIdx.y);
}


// Right-hand factor of the update, scaled: Bp[c + j*ldb] for c < K + nc, j < nc:
//   c <  K : -(S T^{-1})[c, j] * 2^{cexp[c]}      (or -S[c, j] * 2^{cexp[c]} if T is null)
//   c >= K :  T^{-1}[c-K, j]   * 2^{cexp[c]}      (or the identity)
// and the per-column max |Bp| into bmax (bit patterns).
__device__ __forceinline__ void bbuild_body(const double* __restrict__ S, int lds, const double* __restrict__ T,
                                            int ldt, int K, int nc, const int* __restrict__ cexp,
                                            double* __restrict__ Bp, int ldb, unsigned long long* __restrict__ bmax,
                                            int bx) {
    __shared__ double ti[64][65];
    const int tid = threadIdx.x;
    // T^{-1} (upper, nc x nc, nc <= 64): column j solves T y = e_j by back substitution.
    if (T != nullptr) {
        if (tid < nc) {
            const int j = tid;
            for (int i = nc - 1; i >= 0; --i) {
                double v = (i == j) ? 1.0 : 0.0;
                for (int l = i + 1; l <= j; ++l) v -= T[i + (i64)l * ldt] * ti[l][j];
                ti[i][j] = (i <= j) ? v / T[i + (i64)i * ldt] : 0.0;
            }
        }
    } else {
        for (int e = tid; e < 64 * 64; e += blockDim.x) ti[e / 64][e % 64] = (e / 64 == e % 64) ? 1.0 : 0.0;
    }
    __syncthreads();
    const int c = bx * 64 + (tid & 63);
    for (int j = tid >> 6; j < nc; j += 4) {
        double v = 0.0;
        if (c < K) {
            if (T != nullptr) {
                for (int l = 0; l <= j; ++l) v -= S[c + (i64)l * lds] * ti[l][j];
            } else {
                v = -S[c + (i64)j * lds];
            }
        } else if (c < K + nc) {
            v = ti[c - K][j];
        }
        if (c < K + nc) {
            v = ldexp(v, cexp[c]);
            Bp[c + (i64)j * ldb] = v;
            unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFULL;
            if ((b >> 52) == 0x7FF) b = 0;
            atomicMax(bmax + j, b);
        }
    }
}

__global__ void __launch_bounds__(256)
bbuild_kernel(const double* __restrict__ S, int lds, const double* __restrict__ T, int ldt, int K, int nc,
              const int* __restrict__ cexp, double* __restrict__ Bp, int ldb,
              unsigned long long* __restrict__ bmax) {
    bbuild_body(S, lds, T, ldt, K, nc, cexp, Bp, ldb, bmax, (int)blockIdx.x);
}

// Right-hand factor of the fused update of the lagged one-sync variants. With
// Q = X[:, 0:K], U_k = X[:, K:K+s], X_{k+1} = X[:, K+s:K+s+nz] it produces, in one
// product over those K + s + nz columns,
//   Q_k     = (U_k - Q Y) Ty^{-1}                      (columns j < s)
//   U_{k+1} = (X_{k+1} - [Q Q_k] S') Ts^{-1}           (columns s + l, l < nz)
// by substituting Q_k into the second line: with M = Ty^{-1} S'_mid and W = Ts^{-1},
//   rows of Q:        [-Y Ty^{-1}        | (-S'_top + Y M) W]
//   rows of U_k:      [ Ty^{-1}          | -M W             ]
//   rows of X_{k+1}:  [ 0                |  W               ]
// (Y = G[0:K, 0:s], S' = [S'_top; S'_mid] of K + s rows; W = I when Ts is null, the
// unscaled first pass of bcgsi21s). Rows are scaled by 2^cexp[c]; bmax collects
// the column maxima.
__device__ __forceinline__ void bbuild_fused_body(const double* __restrict__ G, int ldg, int K, int s,
                                                  const double* __restrict__ Ty, int ldty,
                                                  const double* __restrict__ Sp, int ldsp,
                                                  const double* __restrict__ Ts, int ldts, int nz,
                                                  const int* __restrict__ cexp, double* __restrict__ Bp, int ldb,
                                                  unsigned long long* __restrict__ bmax, int bx, double* fsm) {
    // Ty^{-1} (s x s), Ts^{-1} (nz x nz) and M (s x nz) in shared memory (fsm),
    // row stride FW = 65 (s, nz <= 64).
    constexpr int FW = 65;
    double* w1 = fsm;
    double* w2 = fsm + 64 * FW;
    double* mm = fsm + 2 * 64 * FW;
#define W1(i, j) w1[(i) * FW + (j)]
#define W2(i, j) w2[(i) * FW + (j)]
#define MM(i, j) mm[(i) * FW + (j)]
    const int tid = threadIdx.x;
    // Ty^{-1} and Ts^{-1} (upper), one column per thread (threads 0..63 and 64..127).
    if (tid < s) {
        const int j = tid;
        for (int i = s - 1; i >= 0; --i) {
            double v = (i == j) ? 1.0 : 0.0;
            for (int l = i + 1; l <= j; ++l) v -= Ty[i + (i64)l * ldty] * W1(l, j);
            W1(i, j) = (i <= j) ? v / Ty[i + (i64)i * ldty] : 0.0;
        }
    } else if (tid >= 64 && tid < 64 + nz) {
        const int j = tid - 64;
        for (int i = nz - 1; i >= 0; --i) {
            double v = (i == j) ? 1.0 : 0.0;
            if (Ts != nullptr) {
                for (int l = i + 1; l <= j; ++l) v -= Ts[i + (i64)l * ldts] * W2(l, j);
                W2(i, j) = (i <= j) ? v / Ts[i + (i64)i * ldts] : 0.0;
            } else {
                W2(i, j) = v;
            }
        }
    }
    __syncthreads();
    // M = Ty^{-1} S'_mid  (s x nz)
    for (int e = tid; e < s * nz; e += blockDim.x) {
        const int a = e % s, l = e / s;
        double v = 0.0;
        for (int b = a; b < s; ++b) v += W1(a, b) * Sp[(K + b) + (i64)l * ldsp];
        MM(a, l) = v;
    }
    __syncthreads();
    const int kin = K + s + nz, nout = s + nz;
    const int c = bx * 64 + (tid & 63);
    if (c >= kin) return;
    for (int j = tid >> 6; j < nout; j += 4) {
        double v = 0.0;
        if (j < s) {
            if (c < K) {
                for (int l = 0; l <= j; ++l) v -= G[c + (i64)l * ldg] * W1(l, j);
            } else if (c < K + s) {
                v = W1(c - K, j);
            }
        } else {
            const int l = j - s;
            if (c < K) {
                for (int q = 0; q <= l; ++q) {
                    double tq = -Sp[c + (i64)q * ldsp];
                    for (int a = 0; a < s; ++a) tq += G[c + (i64)a * ldg] * MM(a, q);
                    v += tq * W2(q, l);
                }
            } else if (c < K + s) {
                for (int q = 0; q <= l; ++q) v -= MM(c - K, q) * W2(q, l);
            } else {
                v = W2(c - K - s, l);
            }
        }
        v = ldexp(v, cexp[c]);
        Bp[c + (i64)j * ldb] = v;
        unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFULL;
        if ((b >> 52) == 0x7FF) b = 0;
        atomicMax(bmax + j, b);
    }
}

__global__ void __launch_bounds__(256)
bbuild_fused_kernel(const double* __restrict__ G, int ldg, int K, int s, const double* __restrict__ Ty,
                    int ldty, const double* __restrict__ Sp, int ldsp, const double* __restrict__ Ts,
                    int ldts, int nz, const int* __restrict__ cexp, double* __restrict__ Bp, int ldb,
                    unsigned long long* __restrict__ bmax) {
    extern __shared__ double fsm[];
    bbuild_fused_body(G, ldg, K, s, Ty, ldty, Sp, ldsp, Ts, ldts, nz, cexp, Bp, ldb, bmax, (int)blockIdx.x, fsm);
}

#undef W1
#undef W2
#undef MM

// Digits of the right-hand factor: bdig[plane][j][c] (K-major), zero padded to
// (NB rows, Kpad columns); fexp[j] = its column scale exponent.
template <int KD>
__device__ __forceinline__ void bdigit_body(const double* __restrict__ Bp, int ldb, int K, int nc, int NB, int Kpad,
                                            const unsigned long long* __restrict__ bmax, int* __restrict__ fexp,
                                            unsigned short* __restrict__ bdig, int bx) {
    const int c = bx * blockDim.x + threadIdx.x;
    if (bx == 0 && threadIdx.x < NB) fexp[threadIdx.x] = threadIdx.x < nc ? scale_exp(bmax[threadIdx.x]) : 0;
    if (c >= Kpad) return;
    for (int j = 0; j < NB; ++j) {
        int d[KD];
        if (c < K + nc && j < nc) {
            split_digits<KD>(Bp[c + (i64)j * ldb], scale_exp(bmax[j]), d);
        } else {
#pragma unroll
            for (int i = 0; i < KD; ++i) d[i] = 0;
        }
#pragma unroll
        for (int i = 0; i < KD; ++i) bdig[((i64)i * NB + j) * Kpad + c] = bf16_bits_of_int(d[i]);
    }
}

template <int KD>
__global__ void __launch_bounds__(256)
bdigit_kernel(const double* __restrict__ Bp, int ldb, int K, int nc, int NB, int Kpad,
              const unsigned long long* __restrict__ bmax, int* __restrict__ fexp,
              unsigned short* __restrict__ bdig) {
    bdigit_body<KD>(Bp, ldb, K, nc, NB, Kpad, bmax, fexp, bdig, (int)blockIdx.x);
}

// ---------------------------------------------------------------------------
// Shared mainloop pieces.
// ---------------------------------------------------------------------------
struct Ring {
    int slot = 0;
    uint32_t phase = 0;
    uint32_t used = 0;   // slots advanced past so far
    __device__ __forceinline__ void advance(int R) {
        ++used;
        if (++slot == R) { slot = 0; phase ^= 1u; }
    }
};

// After an abort, the producer waits (20 ms at most per slot) until the loads of
// the ring slots it armed most recently have landed, so that no copy is still
// writing this CTA's shared memory when it exits. The most recent arming of each
// slot is the one whose phase may still be open.
__device__ __forceinline__ void drain_ring(uint64_t* full, int R, const Ring& r) {
    int slot = r.slot;
    uint32_t phase = r.phase;
    const uint32_t armed = r.used < (uint32_t)R ? r.used : (uint32_t)R;
    for (uint32_t i = 0; i < armed; ++i) {
        if (--slot < 0) { slot = R - 1; phase ^= 1u; }
        tc::mbar_wait_for(&full[slot], phase, 20000000ULL);
    }
}

template <int NB, int KD>
struct SmemLayout {
    static constexpr int B_SLOT = KD * NB * KCH * 2;
    static constexpr int A_OFF = 0;
    static constexpr int B_OFF = RA * A_SLOT;
    static constexpr int BAR_OFF = B_OFF + RB * B_SLOT;
    static constexpr int BYTES = BAR_OFF + 512 + 1024;  // barriers (<= 512 B) + alignment slack
    static constexpr int TMEM_COLS_PER_BUF = NB * KD;
    static constexpr int TMEM_ALLOC = (2 * TMEM_COLS_PER_BUF) <= 128 ? 128 : ((2 * TMEM_COLS_PER_BUF) <= 256 ? 256 : 512);
};

constexpr int RQ = 4;          // tile-number ring depth (update kernel)
struct Bars {
    uint64_t a_full[RA], a_empty[RA], b_full[RB], b_empty[RB], t_full[2], t_empty[2], drain;
    uint64_t q_full[RQ], q_empty[RQ];
};
static_assert(sizeof(Bars) <= 512, "barrier block exceeds its shared-memory reservation");

// acc + a * b, 32 x 32 -> 64-bit signed, in one multiply-add.
__device__ __forceinline__ long long mad_wide(int a, int b, long long acc) {
    long long d;
    asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(acc));
    return d;
}

// Adds TMEM group g's values v[0..NH) into the accumulators (see accumulate_window).
template <int NH>
__device__ __forceinline__ void add_group(int g, const float* v, long long* hi, long long* mid, float* lo) {
    if (g < 3) {
        const int f = 1 << (8 * (2 - g));
#pragma unroll
        for (int q = 0; q < NH; ++q) hi[q] = mad_wide(__float2int_rn(v[q]), f, hi[q]);
    } else if (g < 6) {
        const int f = 1 << (8 * (5 - g));
#pragma unroll
        for (int q = 0; q < NH; ++q) mid[q] = mad_wide(__float2int_rn(v[q]), f, mid[q]);
    } else {
        const float w = __int_as_float((127 - 8 * (g - 6)) << 23);  // 2^{-8(g-6)}
#pragma unroll
        for (int q = 0; q < NH; ++q) lo[q] = fmaf(v[q], w, lo[q]);
    }
}

// Per-window epilogue accumulation of the TMEM groups: groups 0-2 (weights 1,
// 2^-8, 2^-16) into the exact 64-bit integer hi, groups 3-5 into the exact 64-bit
// integer mid (weight 2^-24 relative to hi's unit), and groups >= 6 (weight <=
// 2^-48) into FP32. Group g sums g + 1 digit products of magnitude <= 2^14 per
// summation step; over the 128 steps of a window every partial sum of every group
// stays below 7 * 2^21 < 2^24, so the FP32 accumulation in TMEM is exact. With 8 or 4
// columns per thread the group loads go out in batches (4 groups, or all) under
// one wait each; with 16 (the Gram, not bound by its epilogue) each load waits
// on its own.
template <int NB, int KD, int NH = NB / 2>
__device__ __forceinline__ void accumulate_window(uint32_t taddr, int col0, long long* hi, long long* mid,
                                                  float* lo) {
    if constexpr (NH == 16) {
#pragma unroll
        for (int g = 0; g < KD; ++g) {
            float v[NH];
            tc::tmem_ld16(taddr + (uint32_t)(g * NB + col0), v);
            add_group<NH>(g, v, hi, mid, lo);
        }
    } else {
        static_assert(NH == 8 || NH == 4, "columns per thread");
        constexpr int GB = NH == 8 ? 4 : KD;   // groups per batch of loads (32 or 28 registers)
#pragma unroll
        for (int g0 = 0; g0 < KD; g0 += GB) {
            uint32_t r[GB][NH];
#pragma unroll
            for (int b = 0; b < GB; ++b) {
                if (g0 + b >= KD) break;
                if constexpr (NH == 8) tc::tmem_ld8_nowait(taddr + (uint32_t)((g0 + b) * NB + col0), r[b]);
                else tc::tmem_ld4_nowait(taddr + (uint32_t)((g0 + b) * NB + col0), r[b]);
            }
            tc::tmem_wait_ld();
#pragma unroll
            for (int b = 0; b < GB; ++b) {
                if (g0 + b >= KD) break;
                if constexpr (NH == 8) tc::tmem_tie8(r[b]);
                else tc::tmem_tie4(r[b]);
                float v[NH];
#pragma unroll
                for (int q = 0; q < NH; ++q) v[q] = __uint_as_float(r[b][q]);
                add_group<NH>(g0 + b, v, hi, mid, lo);
            }
        }
    }
}

// The FP64 value (hi * 2^48 + mid * 2^24 + lo * 2^16) * 2^e2, rounded to nearest,
// built with integer operations only (the FP64 pipe of GB300 runs at 2 operations
// per SM per clock, too slow for a per-element epilogue). With the group weights
// hi = D0 2^16 + D1 2^8 + D2, mid = D3 2^16 + D4 2^8 + D5, lo = D6 + D7 2^-8 + ...,
// W = 2^64 * sum_g D_g 2^{-8g}.
__device__ __forceinline__ double assemble(long long hi, long long mid, float lo, int e2) {
    // W as two 64-bit limbs (wh, wl): the three terms sign-extended and added with
    // the carries out of the low limb.
    const long long L = __float2ll_rn(lo * 65536.0f);
    unsigned long long wl = (unsigned long long)hi << 48;
    unsigned long long wh = (unsigned long long)(hi >> 16);
    const unsigned long long ml = (unsigned long long)mid << 24;
    unsigned long long t = wl + ml;
    wh += (unsigned long long)(mid >> 40) + (unsigned long long)(t < wl);
    wl = t;
    t = wl + (unsigned long long)L;
    wh += (unsigned long long)(L >> 63) + (unsigned long long)(t < wl);
    wl = t;
    if ((wl | wh) == 0ULL) return 0.0;
    const unsigned long long sign = wh & 0x8000000000000000ULL;
    if (sign) {   // |W|
        wl = ~wl + 1ULL;
        wh = ~wh + (unsigned long long)(wl == 0ULL);
    }
    // T: the 64 bits of |W| from its leading one (at bit p) down, the leading one
    // at bit 63. The 53-bit mantissa is T >> 11, rounded by bit 10 (half away from
    // zero); below 2^53 T's low bits are zero and nothing rounds.
    int p;
    unsigned long long T;
    if (wh) {
        const int lz = __clzll((long long)wh);
        p = 127 - lz;
        T = lz ? (wh << lz) | (wl >> (64 - lz)) : wh;
    } else {
        const int lz = __clzll((long long)wl);
        p = 63 - lz;
        T = wl << lz;
    }
    unsigned long long mant = (T >> 11) + ((T >> 10) & 1ULL);
    int pe = p;
    if (mant >> 53) { mant >>= 1; ++pe; }
    const int E = pe + e2 + 1023;
    if (E <= 0) return __longlong_as_double((long long)sign);
    if (E >= 2047) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ULL));
    return __longlong_as_double((long long)(sign | ((unsigned long long)E << 52) | (mant & 0xFFFFFFFFFFFFFULL)));
}

// Producer: for each chunk, KD B planes then the KA most significant A planes
// (TMA), each with its L2 eviction policy (polA, polB). The coordinate function also picks the A map
// and the bytes its box holds: the update's last K chunk uses a map whose box
// covers only the chunk's valid columns, so it does not read past kin.
template <int NB, int KD, int KA = KD, class CoordFn>
__device__ __forceinline__ bool produce_chunk(const CUtensorMap* mapB, uint8_t* sA, uint8_t* sB, Bars* bars,
                                              Ring& ra, Ring& rb, CoordFn coords, int item, int ch,
                                              volatile int* abort, int* err, uint64_t polA, uint64_t polB) {
    constexpr int B_SLOT = SmemLayout<NB, KD>::B_SLOT;
    // Plane p of A is at (ax, ay, az + p*azs); plane p of B at (bx, by, bz + p*bzs).
    int ax, ay, az, azs, bx, by, bz, bzs;
    uint32_t abytes;
    const CUtensorMap* mapA;
    coords(item, ch, ax, ay, az, azs, bx, by, bz, bzs, mapA, abytes);
    if (!tc::mbar_wait(&bars->b_empty[rb.slot], rb.phase ^ 1u, abort, err, 11)) return false;
    tc::mbar_expect_tx(&bars->b_full[rb.slot], (uint32_t)B_SLOT);
#pragma unroll
    for (int j = 0; j < KD; ++j)
        tc::tma_load_3d_hint(sB + rb.slot * B_SLOT + j * NB * KCH * 2, mapB, &bars->b_full[rb.slot], bx, by,
                             bz + j * bzs, polB);
    rb.advance(RB);
#pragma unroll
    for (int i = 0; i < KA; ++i) {
        if (!tc::mbar_wait(&bars->a_empty[ra.slot], ra.phase ^ 1u, abort, err, 12 + 100 * ra.slot)) return false;
        tc::mbar_expect_tx(&bars->a_full[ra.slot], abytes);
        tc::tma_load_3d_hint(sA + ra.slot * A_SLOT, mapA, &bars->a_full[ra.slot], ax, ay, az + i * azs, polA);
        ra.advance(RA);
    }
    return true;
}

// MMA issuer for one chunk into TMEM buffer `dcol` (column offset): A plane i
// (i < KA) times B planes 0 .. KD-1-i into TMEM groups i .. KD-1. A_MN: the A
// tile is two 64-row blocks (LBO apart: 8 KB for a whole chunk, kv * 128 bytes
// for a last chunk of kv columns) of K-rows of 128 bytes (MN-major); only the
// first ksteps 16-row K steps are issued.
template <int NB, int KD, bool A_MN = false, int KA = KD>
__device__ __forceinline__ bool mma_chunk(uint32_t tmem_base, uint32_t dcol, uint8_t* sA, uint8_t* sB,
                                          Bars* bars, Ring& ra, Ring& rb, bool first_in_window,
                                          volatile int* abort, int* err, int ksteps = KCH / 16,
                                          uint32_t lbo = 64 * KCH * 2) {
    constexpr int B_SLOT = SmemLayout<NB, KD>::B_SLOT;
    if (!tc::mbar_wait(&bars->b_full[rb.slot], rb.phase, abort, err, 21)) return false;
    const uint32_t b_addr = tc::smem_u32(sB + rb.slot * B_SLOT);
#pragma unroll
    for (int i = 0; i < KA; ++i) {
        if (!tc::mbar_wait(&bars->a_full[ra.slot], ra.phase, abort, err, 22 + 100 * ra.slot)) return false;
        tc::tc_fence_after();
        const uint32_t a_addr = tc::smem_u32(sA + ra.slot * A_SLOT);
        const uint32_t idesc = A_MN ? tc::idesc_bf16_f32_amn(TILE_M, NB * (KD - i))
                                    : tc::idesc_bf16_f32(TILE_M, NB * (KD - i));
#pragma unroll
        for (int k = 0; k < KCH / 16; ++k) {
            if (k >= ksteps) break;
            const uint64_t da = A_MN ? tc::sw128_desc_mn(a_addr + k * 16 * 128, lbo)
                                     : tc::sw128_desc(a_addr + k * 32);
            const uint64_t db = tc::sw128_desc(b_addr + k * 32);
            const uint32_t acc = (first_in_window && i == 0 && k == 0) ? 0u : 1u;
            tc::mma_bf16(tmem_base + dcol + (uint32_t)(i * NB), da, db, idesc, acc);
        }
        tc::mma_commit(&bars->a_empty[ra.slot]);
        ra.advance(RA);
    }
    tc::mma_commit(&bars->b_empty[rb.slot]);
    rb.advance(RB);
    return true;
}

template <int NB, int KD>
__device__ __forceinline__ Bars* setup_cta(uint8_t* smem_raw, uint8_t*& sA, uint8_t*& sB, uint32_t* tmem_slot,
                                           int nepi = NEPI) {
    using L = SmemLayout<NB, KD>;
    uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    sA = base + L::A_OFF;
    sB = base + L::B_OFF;
    Bars* bars = reinterpret_cast<Bars*>(base + L::BAR_OFF);
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int i = 0; i < RA; ++i) { tc::mbar_init(&bars->a_full[i], 1); tc::mbar_init(&bars->a_empty[i], 1); }
        for (int i = 0; i < RB; ++i) { tc::mbar_init(&bars->b_full[i], 1); tc::mbar_init(&bars->b_empty[i], 1); }
        for (int i = 0; i < 2; ++i) { tc::mbar_init(&bars->t_full[i], 1); tc::mbar_init(&bars->t_empty[i], (uint32_t)(nepi / 32)); }
        tc::mbar_init(&bars->drain, 1);
        // Tile-number ring: one producer; the MMA thread and every epilogue warp read.
        for (int i = 0; i < RQ; ++i) { tc::mbar_init(&bars->q_full[i], 1); tc::mbar_init(&bars->q_empty[i], (uint32_t)(1 + nepi / 32)); }
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tmem_slot, (uint32_t)L::TMEM_ALLOC);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    return bars;
}

// ---------------------------------------------------------------------------
// Tall Gram: part[rc][c + j*na] = sum over rows of this CTA's range of
// X[r, c] X[r, b0 + j] for c in the M-block, j in the N-group.
// ---------------------------------------------------------------------------
struct GramParams {
    int na, nb, b0, nrc;
    int a_once;      // 1: every A tile is read by one CTA only (numNG == 1), loaded evict_first
    int alast;       // columns the last M-block's A box holds (na - 128 (numMB - 1), rounded up to 16)
    i64 m;
    int numMB, numNG, rc;
    i64 rows_per;   // multiple of ROW_ALIGN
    const int* cexp;
    double* part;
    int* err;
};

// One Gram of a batched launch: its tensor maps (in global memory) and parameters.
struct SplitGramJob {   // the CUtensorMap members keep the struct 64-byte aligned
    CUtensorMap mapA, mapAlast, mapB;
    GramParams p;
};

// BATCH: the CTAs of many Grams in one launch; CTA b runs item b - prefix[j] of
// job j (prefix[j] <= b < prefix[j + 1]) with job j's maps and parameters, and
// exactly the arithmetic of a single launch of that Gram. p0.err is the launch's.
template <int NB, int KD, int KA, bool BATCH>
__global__ void __launch_bounds__(NTHREADS, 1)
gram_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapAlast,
               const __grid_constant__ CUtensorMap mapB, GramParams p0, const SplitGramJob* __restrict__ jobs,
               const int* __restrict__ prefix, int njobs) {
    using L = SmemLayout<NB, KD>;
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    uint8_t *sA, *sB;
    if (threadIdx.x == 0) abort_flag = 0;
    Bars* bars = setup_cta<NB, KD>(smem_raw, sA, sB, &tmem_slot);
    const uint32_t tmem = tmem_slot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    int item = blockIdx.x;
    GramParams p = p0;
    const CUtensorMap *mA = &mapA, *mAl = &mapAlast, *mB = &mapB;
    if constexpr (BATCH) {
        const int j = batched_job_of(prefix, njobs, item);
        item -= prefix[j];
        p = jobs[j].p;
        p.err = p0.err;
        mA = &jobs[j].mapA; mAl = &jobs[j].mapAlast; mB = &jobs[j].mapB;
        if (threadIdx.x == 0) {   // the producer: maps written by the host before the launch
            tc::fence_tensormap(mA);
            tc::fence_tensormap(mAl);
            tc::fence_tensormap(mB);
        }
    }
    const int mb = item % p.numMB;
    const int ng = (item / p.numMB) % p.numNG;
    const int rcI = item / (p.numMB * p.numNG);
    const i64 r0 = (i64)rcI * p.rows_per;
    const i64 r1 = min(p.m, r0 + p.rows_per);
    const int nchunks = r1 > r0 ? (int)ceil_div(r1 - r0, KCH) : 0;
    const int nwin = (nchunks + WIN - 1) / WIN;

    // The last M-block, when na is not a multiple of 128, loads only its
    // p.alast columns (mapAlast's box); the tile's other rows keep stale data
    // and give D rows that are not written.
    const bool last_part = mb == p.numMB - 1 && p.alast < TILE_M;
    auto coords = [&](int, int ch, int& ax, int& ay, int& az, int& azs, int& bx, int& by, int& bz, int& bzs,
                      const CUtensorMap*& amap, uint32_t& abytes) {
        const int rc = (int)((r0 + (i64)ch * KCH) / KCH);   // 64-row chunk of the column store
        ax = 0; ay = mb * TILE_M; az = rc; azs = p.nrc;
        bx = 0; by = p.b0 + ng * NB; bz = rc; bzs = p.nrc;
        amap = last_part ? mAl : mA;
        abytes = last_part ? (uint32_t)(p.alast * KCH * 2) : (uint32_t)A_SLOT;
    };

    if (warp == 0) {
        if (lane == 0) {
            // The numMB CTAs of one (row range, N-group) read the same B tiles at
            // about the same time: B stays in L2 (evict_last) for the others.
            const uint64_t polA = p.a_once ? tc::policy_evict_first() : tc::policy_evict_normal();
            const uint64_t polB = tc::policy_evict_last();
            Ring ra, rb;
            for (int ch = 0; ch < nchunks; ++ch)
                if (!produce_chunk<NB, KD, KA>(mB, sA, sB, bars, ra, rb, coords, 0, ch, &abort_flag, p.err, polA,
                                               polB))
                    break;
            if (abort_flag) {
                drain_ring(bars->a_full, RA, ra);
                drain_ring(bars->b_full, RB, rb);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            Ring ra, rb;
            bool ok = true;
            for (int w = 0; w < nwin && ok; ++w) {
                const int buf = w & 1;
                const uint32_t tph = (uint32_t)((w >> 1) & 1);
                if (!tc::mbar_wait(&bars->t_empty[buf], tph ^ 1u, &abort_flag, p.err, 31)) break;
                tc::tc_fence_after();
                const int c_end = min(nchunks, (w + 1) * WIN);
                for (int ch = w * WIN; ch < c_end && ok; ++ch)
                    ok = mma_chunk<NB, KD, false, KA>(tmem, (uint32_t)(buf * L::TMEM_COLS_PER_BUF), sA, sB, bars, ra,
                                                      rb, ch == w * WIN, &abort_flag, p.err);
                if (ok) tc::mma_commit(&bars->t_full[buf]);
            }
            tc::mma_commit(&bars->drain);
        }
    } else {
        // Epilogue: two threads per TMEM lane (32*(warp%4) + lane) = A column, each
        // owning half of the NB output columns.
        constexpr int NH = NB / 2;
        const int quarter = warp & 3;
        const int half = (warp - 2) >> 2;
        const int row = quarter * 32 + lane;
        long long hi[NH], mid[NH];
        float lo[NH];
#pragma unroll
        for (int j = 0; j < NH; ++j) { hi[j] = 0; mid[j] = 0; lo[j] = 0.f; }
        bool ok = true;
        for (int w = 0; w < nwin; ++w) {
            const int buf = w & 1;
            const uint32_t tph = (uint32_t)((w >> 1) & 1);
            // Warp-uniform: the TMEM loads below are .sync.aligned.
            const bool got = tc::mbar_wait(&bars->t_full[buf], tph, &abort_flag, p.err, 41);
            if (!__all_sync(0xffffffffu, got)) { ok = false; break; }
            tc::tc_fence_after();
            const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * L::TMEM_COLS_PER_BUF);
            accumulate_window<NB, KD>(taddr, half * NH, hi, mid, lo);
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&bars->t_empty[buf]);   // one arrival per warp
        }
        if (ok && !abort_flag) {
            const int c = mb * TILE_M + row;
            if (c < p.na) {
                const int ec = p.cexp[c];
                double* out = p.part + (i64)rcI * p.na * p.nb;
#pragma unroll
                for (int jj = 0; jj < NH; ++jj) {
                    const int j = ng * NB + half * NH + jj;
                    if (j < p.nb) out[c + (i64)j * p.na] = assemble(hi[jj], mid[jj], lo[jj], ec + p.cexp[p.b0 + j] - 78);
                }
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        // All MMAs issued by this CTA have completed once `drain` fires.
        if (lane == 0) tc::mbar_wait(&bars->drain, 0, &abort_flag, p.err, 51);
        __syncwarp();
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, (uint32_t)L::TMEM_ALLOC);
    }
}

// ---------------------------------------------------------------------------
// Update: X[r, c0 + j] = sum_c A[r, c] Bp[c, j] over c < K + nc, for 128-row
// tiles (persistent over tiles).
// ---------------------------------------------------------------------------
struct UpdateParams {
    i64 m;
    int nrc;      // 64-row chunks of the column store
    int kin;      // K + nc (inner length)
    int nc, c0;
    i64 ld;
    double* X;
    const int* fexp;
    unsigned long long* cmax;   // column max |X[:, c0 + j]| of the written block (bit patterns; the
                                // high word only, which holds the exponent the digit scale uses)
    int* err;
    int* tile_ctr;              // zeroed before the launch; CTAs take row tiles from it
    int kr_last;                // columns the last K chunk's A box holds: kin - 64 (chunks - 1) rounded up to 16
};

// One update of a batched launch: its tensor maps (in global memory) and
// parameters (tile_ctr and err are the launch's).
struct SplitUpdJob {    // the CUtensorMap members keep the struct 64-byte aligned
    CUtensorMap mapA, mapAlast, mapB;
    UpdateParams p;
};

// BATCH: the row tiles of many updates in one persistent launch. Global tile t
// belongs to job j (tprefix[j] <= t < tprefix[j + 1]) as its tile t - tprefix[j];
// every role resolves each tile to its job, and each tile gets exactly the
// arithmetic of a single launch of that update. A CTA takes tiles in increasing
// order, so its jobs come in increasing order too; the epilogue writes a job's
// column maxima when the next job starts.
template <int NB, int KD, bool BATCH>
__global__ void __launch_bounds__(UTHREADS, 1)
update_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapAlast,
                 const __grid_constant__ CUtensorMap mapB, UpdateParams p0, const SplitUpdJob* __restrict__ jobs,
                 const int* __restrict__ tprefix, int njobs) {
    using L = SmemLayout<NB, KD>;
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    uint8_t *sA, *sB;
    if (threadIdx.x == 0) abort_flag = 0;
    Bars* bars = setup_cta<NB, KD>(smem_raw, sA, sB, &tmem_slot, UNEPI);
    const uint32_t tmem = tmem_slot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const int ntiles = BATCH ? tprefix[njobs] : (int)ceil_div(p0.m, TILE_M);
    __shared__ unsigned long long s_cmax[32];
    if (threadIdx.x < 32) s_cmax[threadIdx.x] = 0ULL;
    __syncthreads();

    // Tile t -> its job's parameters and its tile index within the job.
    auto resolve = [&](int t, int& lt, int& job) -> const UpdateParams* {
        if constexpr (BATCH) {
            job = batched_job_of(tprefix, njobs, t);
            lt = t - tprefix[job];
            return &jobs[job].p;
        } else {
            job = 0;
            lt = t;
            return &p0;
        }
    };

    // Row tiles are handed out dynamically: the producer takes the next tile number
    // from the launch's counter and publishes it through the ring s_tile/q_*; the
    // MMA thread and every epilogue warp read the same sequence. A number >= ntiles
    // ends all three loops. Each tile's arithmetic does not depend on which CTA
    // runs it. The last K chunk loads only its kv = kin - ch * KCH columns, rounded
    // up to 16 (a box of kv columns x two 64-row chunks; the second chunk lands
    // kv * 128 bytes after the first), and issues only their MMA K steps.
    __shared__ int s_tile[RQ];
    if (warp == 0) {
        if (lane == 0) {
            // A tiles are read once per launch; the right-hand factor by every CTA.
            const uint64_t polA = tc::policy_evict_first();
            const uint64_t polB = tc::policy_evict_last();
            Ring ra, rb, rq;
            bool ok = true;
            int fenced = -1;
            while (ok) {
                const int tile = atomicAdd(p0.tile_ctr, 1);
                if (!tc::mbar_wait(&bars->q_empty[rq.slot], rq.phase ^ 1u, &abort_flag, p0.err, 15)) break;
                s_tile[rq.slot] = tile;
                tc::mbar_arrive(&bars->q_full[rq.slot]);
                rq.advance(RQ);
                if (tile >= ntiles) break;
                int lt, job;
                const UpdateParams* q = resolve(tile, lt, job);
                const CUtensorMap *mA = &mapA, *mAl = &mapAlast, *mB = &mapB;
                if constexpr (BATCH) {
                    mA = &jobs[job].mapA; mAl = &jobs[job].mapAlast; mB = &jobs[job].mapB;
                    if (job != fenced) {   // maps written by the host before the launch
                        tc::fence_tensormap(mA);
                        tc::fence_tensormap(mAl);
                        tc::fence_tensormap(mB);
                        fenced = job;
                    }
                }
                const int nchunks = (q->kin + KCH - 1) / KCH;
                const int kr_last = q->kr_last;   // 16, 32, 48 (mapAlast's box) or 64
                const int nrc = q->nrc;
                auto coords = [&](int tl, int ch, int& ax, int& ay, int& az, int& azs, int& bx, int& by, int& bz,
                                  int& bzs, const CUtensorMap*& amap, uint32_t& abytes) {
                    ax = 0; ay = ch * KCH; az = 2 * tl; azs = nrc;   // 64 columns x two 64-row chunks
                    bx = ch * KCH; by = 0; bz = 0; bzs = 1;
                    const bool last = ch == nchunks - 1 && kr_last < KCH;
                    amap = last ? mAl : mA;
                    abytes = (uint32_t)((last ? kr_last : KCH) * 256);
                };
                for (int ch = 0; ch < nchunks && ok; ++ch)
                    ok = produce_chunk<NB, KD>(mB, sA, sB, bars, ra, rb, coords, lt, ch, &abort_flag, p0.err, polA,
                                               polB);
            }
            if (abort_flag) {
                drain_ring(bars->a_full, RA, ra);
                drain_ring(bars->b_full, RB, rb);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            Ring ra, rb, rq;
            bool ok = true;
            int wc = 0;  // window counter across tiles
            while (ok) {
                if (!tc::mbar_wait(&bars->q_full[rq.slot], rq.phase, &abort_flag, p0.err, 33)) break;
                const int tile = s_tile[rq.slot];
                tc::mbar_arrive(&bars->q_empty[rq.slot]);
                rq.advance(RQ);
                if (tile >= ntiles) break;
                int lt, job;
                const UpdateParams* q = resolve(tile, lt, job);
                const int nchunks = (q->kin + KCH - 1) / KCH;
                const int nwin = (nchunks + WIN - 1) / WIN;
                const int kr_last = q->kr_last;
                for (int w = 0; w < nwin && ok; ++w, ++wc) {
                    const int buf = wc & 1;
                    const uint32_t tph = (uint32_t)((wc >> 1) & 1);
                    if (!tc::mbar_wait(&bars->t_empty[buf], tph ^ 1u, &abort_flag, p0.err, 32)) { ok = false; break; }
                    tc::tc_fence_after();
                    const int c_end = min(nchunks, (w + 1) * WIN);
                    for (int ch = w * WIN; ch < c_end && ok; ++ch) {
                        const int kr = ch == nchunks - 1 ? kr_last : KCH;
                        ok = mma_chunk<NB, KD, true>(tmem, (uint32_t)(buf * L::TMEM_COLS_PER_BUF), sA, sB, bars, ra,
                                                     rb, ch == w * WIN, &abort_flag, p0.err, kr / 16,
                                                     (uint32_t)(kr * 128));
                    }
                    if (ok) tc::mma_commit(&bars->t_full[buf]);
                }
            }
            tc::mma_commit(&bars->drain);
        }
    } else {
        constexpr int NH = NB / UEPW;   // output columns per thread
        const int quarter = warp & 3;   // TMEM lane quarter this warp may access
        const int half = (warp - 2) >> 2;   // which NH-column part of the row
        const int rloc = quarter * 32 + lane;
        int wc = 0;
        bool ok = true;
        Ring rq;
        // Running max over this thread's rows of the high word of |x| per output
        // column: the digit scale needs only the exponent of the column max, which
        // the high word holds. Reduced over the CTA once, after the last tile (or,
        // in a batched launch, when the job changes).
        uint32_t rmax[NH];
#pragma unroll
        for (int jj = 0; jj < NH; ++jj) rmax[jj] = 0u;
        const UpdateParams* cq = nullptr;   // the job rmax belongs to (batched launches)
        auto flush = [&](const UpdateParams* fq) {
#pragma unroll
            for (int jj = 0; jj < NH; ++jj) {
                uint32_t a = rmax[jj];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const uint32_t b = __shfl_xor_sync(0xffffffffu, a, o);
                    a = a > b ? a : b;
                }
                const int j = half * NH + jj;
                if (lane == 0 && a && j < fq->nc) atomicMax(fq->cmax + fq->c0 + j, (unsigned long long)a << 32);
                rmax[jj] = 0u;
            }
        };
        while (ok) {
            int tile = 0;
            if (lane == 0) {
                if (!tc::mbar_wait(&bars->q_full[rq.slot], rq.phase, &abort_flag, p0.err, 43)) tile = -1;
                else tile = s_tile[rq.slot];
            }
            tile = __shfl_sync(0xffffffffu, tile, 0);
            if (tile < 0) break;
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&bars->q_empty[rq.slot]);
            rq.advance(RQ);
            if (tile >= ntiles) break;
            int lt, job;
            const UpdateParams* q = resolve(tile, lt, job);
            if constexpr (BATCH) {
                if (q != cq) {
                    if (cq) flush(cq);
                    cq = q;
                }
            }
            const int nchunks = (q->kin + KCH - 1) / KCH;
            const int nwin = (nchunks + WIN - 1) / WIN;
            long long hi[NH], mid[NH];
            float lo[NH];
#pragma unroll
            for (int j = 0; j < NH; ++j) { hi[j] = 0; mid[j] = 0; lo[j] = 0.f; }
            for (int w = 0; w < nwin; ++w, ++wc) {
                const int buf = wc & 1;
                const uint32_t tph = (uint32_t)((wc >> 1) & 1);
                // Warp-uniform: the TMEM loads below are .sync.aligned.
                const bool got = tc::mbar_wait(&bars->t_full[buf], tph, &abort_flag, p0.err, 42);
                if (!__all_sync(0xffffffffu, got)) { ok = false; break; }
                tc::tc_fence_after();
                const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * L::TMEM_COLS_PER_BUF);
                accumulate_window<NB, KD, NH>(taddr, half * NH, hi, mid, lo);
                tc::tc_fence_before();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&bars->t_empty[buf]);   // one arrival per warp
            }
            if (__any_sync(0xffffffffu, !ok || abort_flag)) break;
            const i64 r = (i64)lt * TILE_M + rloc;
            double* xr = q->X + r + (i64)q->c0 * q->ld;
#pragma unroll
            for (int jj = 0; jj < NH; ++jj) {
                const int j = half * NH + jj;
                if (j < q->nc && r < q->m) {
                    const double v = assemble(hi[jj], mid[jj], lo[jj], q->fexp[j] - 78);
                    xr[(i64)j * q->ld] = v;
                    uint32_t a = (uint32_t)((unsigned long long)__double_as_longlong(v) >> 32) & 0x7FFFFFFFu;
                    if ((a >> 20) == 0x7FFu) a = 0u;   // Inf/NaN do not set the scale
                    rmax[jj] = a > rmax[jj] ? a : rmax[jj];
                }
            }
        }
        if constexpr (BATCH) {
            if (cq) flush(cq);
        } else {
#pragma unroll
            for (int jj = 0; jj < NH; ++jj) {
                uint32_t a = rmax[jj];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const uint32_t b = __shfl_xor_sync(0xffffffffu, a, o);
                    a = a > b ? a : b;
                }
                const int j = half * NH + jj;
                if (lane == 0 && a && j < p0.nc) atomicMax(&s_cmax[j], (unsigned long long)a << 32);
            }
        }
    }
    __syncthreads();
    if (!BATCH && threadIdx.x < p0.nc && s_cmax[threadIdx.x])
        atomicMax(p0.cmax + p0.c0 + threadIdx.x, s_cmax[threadIdx.x]);
    if (warp == 1) {
        if (lane == 0) tc::mbar_wait(&bars->drain, 0, &abort_flag, p0.err, 52);
        __syncwarp();
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, (uint32_t)L::TMEM_ALLOC);
    }
}

// ---------------------------------------------------------------------------
// Host side: workspace plan, tensor maps, digit freshness.
// ---------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {   // once, thread-safe
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (PFN_cuTensorMapEncodeTiled_v12000)p;
        return (PFN_cuTensorMapEncodeTiled_v12000)nullptr;
    }();
    return fn;
}

// 3-D BF16 map: dims {inner, outer, planes}, strides in bytes, box {64, box_outer, box_planes}.
int make_map3(CUtensorMap* map, void* base, i64 inner, i64 outer, i64 planes, i64 ld_elems,
              i64 plane_elems, int box_outer, int box_planes = 1) {
    auto enc = encode_fn();
    if (!enc) return (int)cudaErrorNotSupported;
    cuuint64_t dims[3] = {(cuuint64_t)inner, (cuuint64_t)outer, (cuuint64_t)planes};
    cuuint64_t strides[2] = {(cuuint64_t)ld_elems * 2, (cuuint64_t)plane_elems * 2};
    cuuint32_t box[3] = {(cuuint32_t)KCH, (cuuint32_t)box_outer, (cuuint32_t)box_planes};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? 0 : (int)cudaErrorInvalidValue;
}

i64 round_up(i64 a, i64 b) { return (a + b - 1) / b * b; }

// Digit planes of the Gram's first operand. The 56-bit form reads all 7 by
// default; ORTH_GB300_SPLIT_GRAM_PLANES=6 makes its Gram read the 6 most
// significant planes of A (B keeps 7): 1/7 fewer A bytes, with A rounded to 48
// bits in the Gram only (the updates keep 56).
int gram_a_planes(int kd) {
    static const int env = [] {
        const char* v = std::getenv("ORTH_GB300_SPLIT_GRAM_PLANES");
        return v ? std::atoi(v) : 0;
    }();
    return (kd == 7 && env == 6) ? 6 : kd;
}

struct Plan {
    // geometry
    double* X = nullptr;
    i64 ld = 0, m = 0;
    int n = 0, num_sms = kNumSMsDefault;
    i64 nrc = 0, kpad = 0;   // 64-row chunks of the column store; n rounded up to 64
    // device buffers (carved from the workspace)
    unsigned short *colstore = nullptr, *bdig = nullptr;
    int *cexp = nullptr, *fexp = nullptr, *err = nullptr, *tile_ctr = nullptr;
    unsigned long long *cmax = nullptr, *bmax = nullptr;
    double *bfull = nullptr, *part = nullptr;
    i64 part_doubles = 0;
    // maps
    CUtensorMap map_col_a, map_col_b, map_col_b16, map_col_u, map_bdig16, map_bdig32;
    CUtensorMap map_col_a_part[7];   // Gram A boxes of 16, 32, ..., 112 columns (a partial last M-block)
    CUtensorMap map_col_u_part[3];   // update A boxes of 16, 32, 48 columns x two 64-row chunks
    int kd = 7;
    std::vector<char> fresh;
    std::vector<char> cmax_valid;   // cmax[c] already holds max |X[:, c]| (set by the update)
    const void* zeroed_base = nullptr;   // stores zeroed for this base and shape
    i64 zeroed_m = -1;
    int zeroed_n = -1;
};
// One plan per scratch slot (split-precision batches run several at once on
// separate streams); slot 0 serves every single-matrix entry point.
constexpr int kPlanSlots = 16;
Plan g_plans[kPlanSlots];
thread_local int g_plan_slot = 0;
inline Plan& cur_plan() { return g_plans[g_plan_slot]; }

struct Carve {
    char* p;
    size_t off = 0;
    template <class T>
    T* take(i64 count) {
        off = (off + 1023) & ~(size_t)1023;
        T* r = reinterpret_cast<T*>(p + off);
        off += (size_t)count * sizeof(T);
        return r;
    }
};

i64 gram_part_doubles(i64 m, int n, int s, int num_sms) {
    i64 best = 0;
    for (int na = 1; na <= n; na += 1) {
        const int nb = 2 * s;
        const i64 mbn = ceil_div(na, TILE_M) * ceil_div(nb, 32);
        const i64 rc = (i64)num_sms / mbn > 0 ? (i64)num_sms / mbn : 1;
        const i64 v = rc * (i64)na * nb;
        if (v > best) best = v;
    }
    (void)m;
    return best + 1024;
}

size_t layout_bytes(i64 m, int n, int s, int num_sms, Plan* out, char* base) {
    Carve cv{base};
    const i64 nrc = ceil_div(m, 64), kpad = round_up(n, 64);
    unsigned short* col = cv.take<unsigned short>((i64)KD_MAX * nrc * n * 64);
    unsigned short* bd = cv.take<unsigned short>((i64)KD_MAX * 32 * kpad);
    int* cexp = cv.take<int>(n + 64);
    int* fexp = cv.take<int>(64);
    int* err = cv.take<int>(16);
    int* tctr = cv.take<int>(16);
    unsigned long long* cmax = cv.take<unsigned long long>(n + 64);
    unsigned long long* bmax = cv.take<unsigned long long>(128);
    double* bfull = cv.take<double>(kpad * 128);
    const i64 pd = gram_part_doubles(m, n, s, num_sms);
    double* part = cv.take<double>(pd);
    if (out) {
        out->nrc = nrc; out->kpad = kpad;
        out->colstore = col; out->bdig = bd;
        out->cexp = cexp; out->fexp = fexp; out->err = err; out->tile_ctr = tctr;
        out->cmax = cmax; out->bmax = bmax; out->bfull = bfull; out->part = part;
        out->part_doubles = pd;
    }
    return cv.off + 1024;
}

template <class K>
int set_smem(K kernel, int bytes) {
    return smem_attr((const void*)kernel, bytes);
}

int ensure_fresh(int c_begin, int c_end, cudaStream_t st) {
    Plan& P = cur_plan();
    int c = c_begin;
    while (c < c_end) {
        if (P.fresh[c]) { ++c; continue; }
        int e = c;
        while (e < c_end && !P.fresh[e] && e - c < 32 && P.cmax_valid[e] == P.cmax_valid[c]) ++e;
        const int nc = e - c;
        if (!P.cmax_valid[c]) {
            cudaError_t ce = (cudaError_t)zero_async(P.cmax + c, (size_t)nc * sizeof(unsigned long long), st);
            if (ce != cudaSuccess) return (int)ce;
            dim3 g1((unsigned)ceil_div(P.m, 4096), (unsigned)nc);
            colmax_kernel<<<g1, 256, 0, st>>>(P.X, P.ld, P.m, c, P.cmax);
            g_launch_count += 1;
        }
        const dim3 sgrid((unsigned)ceil_div(P.m, 128), (unsigned)ceil_div(nc, 16));
        if (P.kd == 6)
            slice_kernel<6><<<sgrid, 128, 0, st>>>(P.X, P.ld, P.m, P.n, c, nc, P.cmax, P.cexp, P.colstore, P.nrc);
        else
            slice_kernel<7><<<sgrid, 128, 0, st>>>(P.X, P.ld, P.m, P.n, c, nc, P.cmax, P.cexp, P.colstore, P.nrc);
        g_launch_count += 1;
        for (int k = c; k < e; ++k) { P.fresh[k] = 1; P.cmax_valid[k] = 0; }
        c = e;
    }
    return (int)cudaGetLastError();
}

}  // namespace

bool split_supported(i64 m, int n, int s) { return s >= 1 && s <= 64 && n >= 2 * s && m >= TILE_M; }

i64 split_workspace_bytes(i64 m, int n, int s, int num_sms) {
    return (i64)layout_bytes(m, n, s, num_sms, nullptr, nullptr);
}

int split_begin(double* X, i64 ld, i64 m, int n, int s, int kd, char* ws, size_t ws_bytes, int num_sms,
                cudaStream_t st) {
    Plan& P = cur_plan();
    if (kd != 6 && kd != 7) return (int)cudaErrorInvalidValue;
    P.kd = kd;
    const size_t need = layout_bytes(m, n, s, num_sms, &P, ws);
    if (need > ws_bytes) return (int)cudaErrorInvalidValue;
    P.X = X; P.ld = ld; P.m = m; P.n = n; P.num_sms = num_sms;
    P.fresh.assign((size_t)n, 0);
    P.cmax_valid.assign((size_t)n, 0);
    // The store is zeroed whenever the workspace or the shape changes. The chunk
    // padding the slicing never writes (rows past m in the last 64-row chunk) lies
    // inside the TMA boxes and must read as zero. The rest must hold digits or
    // zeros (never bytes of another layout): the last K chunk of an update reads
    // columns past K + nc, multiplied by zero rows of the factor, and the last row
    // tile of an update may read the 64-row chunk after the last one (the next
    // plane's first chunk), whose products land only in rows past m. Repeated runs
    // of one shape keep their zeroed padding.
    if (P.zeroed_base != (const void*)P.colstore || P.zeroed_m != m || P.zeroed_n != n) {
        cudaError_t ce = (cudaError_t)zero_async(P.colstore, (size_t)KD_MAX * P.nrc * 64 * n * 2, st);
        if (ce != cudaSuccess) return (int)ce;
        P.zeroed_base = P.colstore;
        P.zeroed_m = m;
        P.zeroed_n = n;
    }
    cudaError_t ce = (cudaError_t)zero_async(P.err, sizeof(int), st);
    if (ce != cudaSuccess) return (int)ce;
    // Chunked stores as 3-D tensors {64, columns or rows, plane x chunk}.
    int rc = make_map3(&P.map_col_a, P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, TILE_M);
    if (!rc) rc = make_map3(&P.map_col_b, P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, 32);
    if (!rc) rc = make_map3(&P.map_col_b16, P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, 16);
    // Update A tiles: 64 columns of two adjacent 64-row chunks (128 rows).
    if (!rc) rc = make_map3(&P.map_col_u, P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, KCH, 2);
    // Partial boxes: a Gram's last M-block of fewer than 128 columns, an update's
    // last K chunk of fewer than 64 (in 16-column steps).
    for (int q = 0; q < 7 && !rc; ++q)
        rc = make_map3(&P.map_col_a_part[q], P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, 16 * (q + 1));
    for (int q = 0; q < 3 && !rc; ++q)
        rc = make_map3(&P.map_col_u_part[q], P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, 16 * (q + 1), 2);
    if (!rc) rc = make_map3(&P.map_bdig16, P.bdig, P.kpad, 16, KD_MAX, P.kpad, 16 * P.kpad, 16);
    if (!rc) rc = make_map3(&P.map_bdig32, P.bdig, P.kpad, 32, KD_MAX, P.kpad, 32 * P.kpad, 32);
    if (rc) return rc;
    // Shared-memory limits of the tensor-core kernels on this device.
    rc = set_smem(gram_tc_kernel<32, 6, 6, false>, SmemLayout<32, 6>::BYTES);
    if (!rc) rc = set_smem(gram_tc_kernel<32, 7, 7, false>, SmemLayout<32, 7>::BYTES);
    if (!rc) rc = set_smem(gram_tc_kernel<32, 7, 6, false>, SmemLayout<32, 7>::BYTES);
    if (!rc) rc = set_smem(gram_tc_kernel<16, 6, 6, false>, SmemLayout<16, 6>::BYTES);
    if (!rc) rc = set_smem(gram_tc_kernel<16, 7, 7, false>, SmemLayout<16, 7>::BYTES);
    if (!rc) rc = set_smem(gram_tc_kernel<16, 7, 6, false>, SmemLayout<16, 7>::BYTES);
    if (!rc) rc = set_smem(update_tc_kernel<16, 6, false>, SmemLayout<16, 6>::BYTES);
    if (!rc) rc = set_smem(update_tc_kernel<16, 7, false>, SmemLayout<16, 7>::BYTES);
    if (!rc) rc = set_smem(update_tc_kernel<32, 6, false>, SmemLayout<32, 6>::BYTES);
    if (!rc) rc = set_smem(update_tc_kernel<32, 7, false>, SmemLayout<32, 7>::BYTES);
    return rc;
}

void split_mark_stale(int c0, int nc) {
    for (int c = c0; c < c0 + nc && c < (int)cur_plan().fresh.size(); ++c) {
        cur_plan().fresh[c] = 0;
        cur_plan().cmax_valid[c] = 0;
    }
}

// The workspaces were freed: a new one may come back at the same address, so no
// plan may treat its stores as already zeroed.
void split_forget_workspaces() {
    for (Plan& P : g_plans) {
        P.zeroed_base = nullptr;
        P.zeroed_m = -1;
        P.zeroed_n = -1;
    }
}

void split_select_slot(int slot) { g_plan_slot = (slot >= 0 && slot < kPlanSlots) ? slot : 0; }

int* split_error_ptr() { return cur_plan().err; }

int g_last_split_error = 0;

int split_error_word(int* out, cudaStream_t st) {
    cudaError_t ce = cudaMemcpyAsync(out, cur_plan().err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce == cudaSuccess && *out) g_last_split_error = *out;
    return (int)ce;
}

int split_last_error() { return g_last_split_error; }

int split_prepare(int c_end, cudaStream_t st) { return ensure_fresh(0, c_end, st); }

int split_slice_columns(const double* X, i64 ld, i64 m, int n, int kd, unsigned short* digits, int* cexp,
                        unsigned long long* cmax, cudaStream_t st) {
    if ((kd != 6 && kd != 7) || m < 1 || n < 1 || n > 65535) return (int)cudaErrorInvalidValue;
    const i64 nrc = ceil_div(m, 64);
    // The slicing writes rows below m only; the rows past m in the last chunk
    // read as zero, as in the store.
    int rc = zero_async(digits, (size_t)kd * nrc * 64 * n * sizeof(unsigned short), st);
    if (!rc) rc = zero_async(cmax, (size_t)n * sizeof(unsigned long long), st);
    if (rc) return rc;
    colmax_kernel<<<dim3((unsigned)ceil_div(m, 4096), (unsigned)n), 256, 0, st>>>(X, ld, m, 0, cmax);
    const dim3 sgrid((unsigned)ceil_div(m, 128), (unsigned)ceil_div(n, 16));
    if (kd == 6)
        slice_kernel<6><<<sgrid, 128, 0, st>>>(X, ld, m, n, 0, n, cmax, cexp, digits, nrc);
    else
        slice_kernel<7><<<sgrid, 128, 0, st>>>(X, ld, m, n, 0, n, cmax, cexp, digits, nrc);
    g_launch_count += 2;
    return (int)cudaGetLastError();
}

int split_digits() { return cur_plan().kd; }

int launch_gram_split(const double* X, i64 ld, i64 m, int na, int b0, int nb, double* out, int ldo,
                      char* ws, size_t ws_bytes, int num_sms, cudaStream_t st) {
    (void)X; (void)ld; (void)ws; (void)ws_bytes;
    Plan& P = cur_plan();
    if (na <= 0 || nb <= 0) return 0;
    int rc = ensure_fresh(0, na > b0 + nb ? na : b0 + nb, st);
    if (rc) return rc;
    GramParams gp;
    gp.na = na; gp.nb = nb; gp.b0 = b0; gp.m = m;
    const int NB = nb <= 16 ? 16 : 32;   // a 16-column N group for narrow B (blocks of s <= 8)
    gp.numMB = (int)ceil_div(na, TILE_M);
    gp.numNG = (int)ceil_div(nb, NB);
    const int mbn = gp.numMB * gp.numNG;
    gp.rc = num_sms / mbn > 0 ? num_sms / mbn : 1;
    gp.rows_per = round_up(ceil_div(m, gp.rc), (i64)ROW_ALIGN);
    gp.rc = (int)ceil_div(m, gp.rows_per);
    gp.nrc = (int)P.nrc;
    gp.cexp = P.cexp;
    gp.part = P.part;
    gp.err = P.err;
    if ((i64)gp.rc * na * nb > P.part_doubles) return (int)cudaErrorInvalidValue;
    // One wave of CTAs: numMB x numNG per row range. The numMB CTAs of one
    // (row range, N-group) are consecutive in blockIdx.x, so they run at the
    // same time and share each B tile through L2.
    gp.a_once = gp.numNG == 1 ? 1 : 0;
    gp.alast = (int)round_up(na - (i64)(gp.numMB - 1) * TILE_M, 16);
    const CUtensorMap& alast_map = gp.alast < TILE_M ? P.map_col_a_part[gp.alast / 16 - 1] : P.map_col_a;
    const unsigned grid = (unsigned)(mbn * gp.rc);
    const CUtensorMap& bmap = NB == 16 ? P.map_col_b16 : P.map_col_b;
    const int ka = gram_a_planes(P.kd);
#define BCGS_GRAM(NBT, KDT, KAT)                                                                                  \
    gram_tc_kernel<NBT, KDT, KAT, false><<<grid, NTHREADS, SmemLayout<NBT, KDT>::BYTES, st>>>(                \
        P.map_col_a, alast_map, bmap, gp, nullptr, nullptr, 0)
    if (NB == 16) {
        if (P.kd == 6) BCGS_GRAM(16, 6, 6); else if (ka == 6) BCGS_GRAM(16, 7, 6); else BCGS_GRAM(16, 7, 7);
    } else {
        if (P.kd == 6) BCGS_GRAM(32, 6, 6); else if (ka == 6) BCGS_GRAM(32, 7, 6); else BCGS_GRAM(32, 7, 7);
    }
#undef BCGS_GRAM
    g_launch_count += 1;
    rc = (int)cudaGetLastError();
    if (rc) return rc;
    return launch_gram_reduce(P.part, gp.rc, na, nb, out, ldo, st);
}

// bdigit + the tensor-core product X[:, c0:c0+nc] = digits[:, 0:kin] * Bp, after the
// caller has filled Bp/bmax.
// Output columns go in groups of at most 32 (one tensor-core pass each). Every
// group reads the same digit planes of X[:, 0:kin], which were sliced before the
// first group wrote anything, and its own 32 columns of the factor in Bp.
static int finish_update(double* X, i64 ld, i64 m, int kin, int c0, int nc, int num_sms, cudaStream_t st) {
    Plan& P = cur_plan();
    for (int j0 = 0; j0 < nc; j0 += 32) {
        const int ng = nc - j0 < 32 ? nc - j0 : 32;
        const int NB = ng <= 16 ? 16 : 32;
        const double* Bg = P.bfull + (i64)j0 * P.kpad;
        if (P.kd == 6)
            bdigit_kernel<6><<<(unsigned)ceil_div(P.kpad, 256), 256, 0, st>>>(Bg, (int)P.kpad, kin - ng, ng, NB,
                                                                               (int)P.kpad, P.bmax + j0, P.fexp,
                                                                               P.bdig);
        else
            bdigit_kernel<7><<<(unsigned)ceil_div(P.kpad, 256), 256, 0, st>>>(Bg, (int)P.kpad, kin - ng, ng, NB,
                                                                               (int)P.kpad, P.bmax + j0, P.fexp,
                                                                               P.bdig);
        cudaError_t ce = (cudaError_t)zero_async(P.cmax + c0 + j0, (size_t)ng * sizeof(unsigned long long), st);
        if (ce != cudaSuccess) return (int)ce;
        UpdateParams up;
        up.nrc = (int)P.nrc;
        up.m = m; up.kin = kin; up.nc = ng; up.c0 = c0 + j0; up.ld = ld; up.X = X; up.fexp = P.fexp;
        up.cmax = P.cmax; up.err = P.err; up.tile_ctr = P.tile_ctr;
        up.kr_last = (int)round_up(kin - (i64)(ceil_div(kin, KCH) - 1) * KCH, 16);
        const CUtensorMap& ulast_map = up.kr_last < KCH ? P.map_col_u_part[up.kr_last / 16 - 1] : P.map_col_u;
        ce = (cudaError_t)zero_async(P.tile_ctr, sizeof(int), st);
        if (ce != cudaSuccess) return (int)ce;
        const int ntiles = (int)ceil_div(m, TILE_M);
        const int grid = ntiles < num_sms ? ntiles : num_sms;
#define BCGS_UPD(NBT, KDT) \
        update_tc_kernel<NBT, KDT, false><<<grid, UTHREADS, SmemLayout<NBT, KDT>::BYTES, st>>>(                 \
            P.map_col_u, ulast_map, P.map_bdig##NBT, up, nullptr, nullptr, 0)
        if (NB == 16) {
            if (P.kd == 6) BCGS_UPD(16, 6); else BCGS_UPD(16, 7);
        } else {
            if (P.kd == 6) BCGS_UPD(32, 6); else BCGS_UPD(32, 7);
        }
#undef BCGS_UPD
        g_launch_count += 2;
    }
    for (int c = c0; c < c0 + nc; ++c) { P.fresh[c] = 0; P.cmax_valid[c] = 1; }
    return (int)cudaGetLastError();
}

int launch_update_split(double* X, i64 ld, i64 m, int K, int c0, int nc, const double* S, int lds,
                        const double* T, int ldt, char* ws, size_t ws_bytes, int num_sms, cudaStream_t st) {
    (void)ws; (void)ws_bytes;
    Plan& P = cur_plan();
    if (nc <= 0) return 0;
    if (c0 != K || nc > 64 || X != P.X) return (int)cudaErrorInvalidValue;
    int rc = ensure_fresh(0, K + nc, st);
    if (rc) return rc;
    cudaError_t ce = (cudaError_t)zero_async(P.bmax, 64 * sizeof(unsigned long long), st);
    if (ce != cudaSuccess) return (int)ce;
    const int kin = K + nc;
    bbuild_kernel<<<(unsigned)ceil_div(kin, 64), 256, 0, st>>>(S, lds, T, ldt, K, nc, P.cexp, P.bfull,
                                                                  (int)P.kpad, P.bmax);
    g_launch_count += 1;
    return finish_update(X, ld, m, kin, c0, nc, num_sms, st);
}

int launch_fused_update_split(double* X, i64 ld, i64 m, int K, int s, int nz, const double* G, int ldg,
                              const double* Ty, const double* Sp, int ldsp, const double* Ts, int num_sms,
                              cudaStream_t st) {
    Plan& P = cur_plan();
    const int kin = K + s + nz, nout = s + nz;
    if (s > 64 || nz > 64 || X != P.X) return (int)cudaErrorInvalidValue;
    int rc = ensure_fresh(0, kin, st);
    if (rc) return rc;
    cudaError_t ce = (cudaError_t)zero_async(P.bmax, 128 * sizeof(unsigned long long), st);
    if (ce != cudaSuccess) return (int)ce;
    const int fattr_rc = set_smem(bbuild_fused_kernel, (int)(3 * 64 * 65 * sizeof(double)));
    if (fattr_rc) return fattr_rc;
    bbuild_fused_kernel<<<(unsigned)ceil_div(kin, 64), 256, 3 * 64 * 65 * sizeof(double), st>>>(G, ldg, K, s, Ty, s, Sp, ldsp, Ts, nz, nz,
                                                                        P.cexp, P.bfull, (int)P.kpad, P.bmax);
    g_launch_count += 1;
    return finish_update(X, ld, m, kin, K, nout, num_sms, st);
}

// ===========================================================================
// Staged split-precision batches: many independent BCGSI+P-1S QRs (the
// reference's bcgsi2P1s, SRC/orth.c:48-222, on each matrix) in the split form,
// with one launch per stage for all matrices of a wave.
//
// A wave is a set of matrices whose digit stores (14 bytes per element) and
// scratch fit in the plan's device buffer together. For every matrix the planner
// replays the single-matrix split driver's schedule (the TSQR of block 1, then per
// block step: slicing of stale columns, the tensor-core Gram and its fixed-order
// reduction, the small FP64 operations, the right-hand factor, its digits and the
// fused tensor-core update), recording each primitive's parameters exactly as the
// single-matrix launchers compute them (row ranges, chunk counts, digit freshness,
// scales). Every phase then becomes one batched launch over all matrices that have
// it, and each wave is captured as one CUDA graph. Each matrix gets the arithmetic
// of a single run: results are bit-identical to orth_gb300_run_dev in split mode.
// ===========================================================================
namespace {

struct ColmaxJob {
    const double* X;
    i64 ld, m;
    int c0, nrb;
    unsigned long long* cmax;
};
struct SliceJob {
    const double* X;
    i64 ld, m, nrc;
    int n, c0, nc, ntile;
    const unsigned long long* cmax;
    int* cexp;
    unsigned short* colstore;
};
struct BbuildJob {
    int fused;
    const double *S, *T, *G, *Ty, *Sp, *Ts;
    int lds, ldt, ldg, ldsp, K, nc, s, nz;
    const int* cexp;
    double* Bp;
    int ldb;
    unsigned long long* bmax;
};
struct BdigitJob {
    const double* Bp;
    int ldb, K, nc, NB, Kpad;
    const unsigned long long* bmax;
    int* fexp;
    unsigned short* bdig;
};
struct ZeroJob {
    void* p;
    int bytes;
};

__global__ void __launch_bounds__(256)
colmax_batched(const ColmaxJob* __restrict__ jobs, const int* __restrict__ prefix, int njobs) {
    const int j = batched_job_of(prefix, njobs, blockIdx.x);
    const ColmaxJob& J = jobs[j];
    const int it = blockIdx.x - prefix[j];
    colmax_body(J.X, J.ld, J.m, J.c0 + it / J.nrb, it % J.nrb, J.cmax);
}

template <int KD>
__global__ void __launch_bounds__(128, 6)
slice_batched(const SliceJob* __restrict__ jobs, const int* __restrict__ prefix, int njobs) {
    const int j = batched_job_of(prefix, njobs, blockIdx.x);
    const SliceJob& J = jobs[j];
    const int it = blockIdx.x - prefix[j];
    slice_body<KD>(J.X, J.ld, J.m, J.n, J.c0, J.nc, J.cmax, J.cexp, J.colstore, J.nrc, it % J.ntile, it / J.ntile);
}

__global__ void __launch_bounds__(256)
bbuild_batched(const BbuildJob* __restrict__ jobs, const int* __restrict__ prefix, int njobs) {
    extern __shared__ double fsm[];
    const int j = batched_job_of(prefix, njobs, blockIdx.x);
    const BbuildJob& J = jobs[j];
    const int it = blockIdx.x - prefix[j];
    if (J.fused)
        bbuild_fused_body(J.G, J.ldg, J.K, J.s, J.Ty, J.s, J.Sp, J.ldsp, J.Ts, J.nz, J.nz, J.cexp, J.Bp, J.ldb,
                          J.bmax, it, fsm);
    else
        bbuild_body(J.S, J.lds, J.T, J.ldt, J.K, J.nc, J.cexp, J.Bp, J.ldb, J.bmax, it);
}

template <int KD>
__global__ void __launch_bounds__(256)
bdigit_batched(const BdigitJob* __restrict__ jobs, const int* __restrict__ prefix, int njobs) {
    const int j = batched_job_of(prefix, njobs, blockIdx.x);
    const BdigitJob& J = jobs[j];
    bdigit_body<KD>(J.Bp, J.ldb, J.K, J.nc, J.NB, J.Kpad, J.bmax, J.fexp, J.bdig, blockIdx.x - prefix[j]);
}

__global__ void __launch_bounds__(256) zero_list(const ZeroJob* __restrict__ jobs) {
    const ZeroJob& J = jobs[blockIdx.x];
    unsigned char* p = static_cast<unsigned char*>(J.p);
    for (int i = threadIdx.x; i < J.bytes; i += blockDim.x) p[i] = 0;
}

// Copies the batch's error word into every matrix's status slot [4].
__global__ void spread_error(const int* __restrict__ err, int* __restrict__ dstatus, int count) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < count) dstatus[8 * (i64)b + 4] = *err;
}

constexpr size_t kBbuildSmem = 3 * 64 * 65 * sizeof(double);

enum SKind {
    kSZero, kSColmax, kSSlice, kSGram, kSGram16, kSReduce, kSSmall, kSBbuild, kSBdigit, kSUpdate, kSUpdate16, kSTile, kSRoot,
    kSApply,
    kSZeroBuf
};
struct SLaunch {
    int kind;
    size_t job_off, prefix_off;
    int njobs, items;
    i64 bytes;   // kSZeroBuf
};

struct SBlob {
    std::vector<char> bytes;
    template <class T>
    size_t put(const std::vector<T>& v) {
        size_t off = (bytes.size() + 127) & ~(size_t)127;
        bytes.resize(off + v.size() * sizeof(T));
        if (!v.empty()) std::memcpy(bytes.data() + off, v.data(), v.size() * sizeof(T));
        return off;
    }
};

// One matrix of a staged batch.
struct SMat {
    int b;
    i64 m, ld;
    int n, s, p;
    double* X;
    double* R;
    int ldR;
    int* status;
    size_t off = 0, bytes = 0;   // its region of the wave buffer
    Plan P;                      // digit store, maps and freshness (as a single run's)
    double *G1 = nullptr, *G2 = nullptr, *Scol = nullptr, *Sd = nullptr, *Yd = nullptr, *tsqr = nullptr;
};

i64 smat_small_doubles(int n, int s) { return 2LL * (n + s) * 2 * s + (i64)n * s + 3LL * s * s + 64; }

// Bytes of one matrix's region of the wave buffer (digit store, factor, Gram
// partials, FP64 small blocks, TSQR stack); with base != nullptr also carves it.
size_t smat_layout(SMat& M, int num_sms, char* base) {
    size_t off = layout_bytes(M.m, M.n, M.s, num_sms, &M.P, base);
    off = (off + 1023) & ~(size_t)1023;
    double* sb = base ? reinterpret_cast<double*>(base + off) : nullptr;
    off += (size_t)smat_small_doubles(M.n, M.s) * sizeof(double);
    off = (off + 1023) & ~(size_t)1023;
    double* tw = base ? reinterpret_cast<double*>(base + off) : nullptr;
    off += (size_t)tsqr_workspace_doubles(M.m, M.s) * sizeof(double);
    if (base) {
        const int n = M.n, s = M.s;
        M.G1 = sb;
        M.G2 = M.G1 + (i64)(n + s) * 2 * s;
        M.Scol = M.G2 + (i64)(n + s) * 2 * s;
        double* S0 = M.Scol + (i64)n * s;
        M.Sd = S0 + (i64)s * s;
        M.Yd = M.Sd + (i64)s * s;
        M.tsqr = tw;
    }
    return off + 1024;
}

struct SWave {
    std::vector<int> mats;       // indices into SplitStaged::mats
    std::vector<SLaunch> launches;
    SBlob blob;
    void* blob_dev = nullptr;
    size_t used = 0;             // bytes of the wave buffer this wave uses
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;
};

}  // namespace

struct SplitStaged {
    int count = 0, kd = 7, num_sms = kNumSMsDefault;
    std::vector<SMat> mats;
    std::vector<SWave> waves;
    char* buf = nullptr;          // the wave buffer (reused by every wave)
    size_t buf_bytes = 0;
    int* dstatus = nullptr;       // 8 ints per matrix (not owned)
    int* derr = nullptr;          // the batch's split-kernel error word; dtile follows it
    int* dtile = nullptr;
    cudaStream_t own = nullptr;
    long long kernels = 0;
    int nodes = 0;
    bool device = true;           // false: a dry run (no GPU memory)
};

namespace {

// Plans one wave: replays the single-matrix split driver (Engine + run_lagged_fused
// with pyth = true) for each matrix and groups its primitives into phases.
int plan_wave(SplitStaged& S, SWave& W) {
    const int KD = S.kd;
    size_t off = 0;
    for (int i : W.mats) {
        SMat& M = S.mats[i];
        M.off = off;
        char* base = S.device ? S.buf + off : nullptr;
        M.bytes = smat_layout(M, S.num_sms, base);
        off += (M.bytes + 4095) & ~(size_t)4095;
        Plan& P = M.P;
        P.kd = KD;
        P.X = M.X; P.ld = M.ld; P.m = M.m; P.n = M.n; P.num_sms = S.num_sms;
        P.fresh.assign((size_t)M.n, 0);
        P.cmax_valid.assign((size_t)M.n, 0);
        if (S.device) {
            const int n = M.n;
            int rc = make_map3(&P.map_col_a, P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, TILE_M);
            if (!rc) rc = make_map3(&P.map_col_b, P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, 32);
            if (!rc) rc = make_map3(&P.map_col_b16, P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, 16);
            if (!rc) rc = make_map3(&P.map_col_u, P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, KCH, 2);
            for (int q = 0; q < 7 && !rc; ++q)
                rc = make_map3(&P.map_col_a_part[q], P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, 16 * (q + 1));
            for (int q = 0; q < 3 && !rc; ++q)
                rc = make_map3(&P.map_col_u_part[q], P.colstore, 64, n, KD_MAX * P.nrc, 64, (i64)n * 64, 16 * (q + 1),
                               2);
            if (!rc) rc = make_map3(&P.map_bdig16, P.bdig, P.kpad, 16, KD_MAX, P.kpad, 16 * P.kpad, 16);
            if (!rc) rc = make_map3(&P.map_bdig32, P.bdig, P.kpad, 32, KD_MAX, P.kpad, 32 * P.kpad, 32);
            if (rc) return rc;
        }
    }
    W.used = off;
    W.launches.clear();
    W.blob.bytes.clear();
    // The store must read as zero where nothing is sliced (rows past m in the
    // last 64-row chunk feed the Gram's sums) and hold no NaN bit patterns where a
    // box reads past its columns: the wave's region is cleared first.
    if (S.device) W.launches.push_back({kSZeroBuf, 0, 0, 0, 0, (i64)off});

    auto push = [&](int kind, auto& jobs, const std::vector<int>& counts) {
        if (jobs.empty()) return;
        std::vector<int> prefix(jobs.size() + 1, 0);
        for (size_t j = 0; j < jobs.size(); ++j) prefix[j + 1] = prefix[j] + counts[j];
        SLaunch L{kind, W.blob.put(jobs), W.blob.put(prefix), (int)jobs.size(), prefix.back(), 0};
        if (L.items > 0) W.launches.push_back(L);
    };
    auto push_zero = [&](std::vector<ZeroJob>& z) {
        if (z.empty()) return;
        SLaunch L{kSZero, W.blob.put(z), 0, (int)z.size(), (int)z.size(), 0};
        W.launches.push_back(L);
    };

    std::vector<ZeroJob> zj;
    std::vector<ColmaxJob> cj;
    std::vector<int> cc;
    std::vector<SliceJob> sj;
    std::vector<int> sc;
    auto flush_prepare = [&]() {
        push_zero(zj);
        push(kSColmax, cj, cc);
        push(kSSlice, sj, sc);
        zj.clear(); cj.clear(); cc.clear(); sj.clear(); sc.clear();
    };
    // ensure_fresh of one matrix, as jobs.
    auto prepare = [&](SMat& M, int c_end) {
        Plan& P = M.P;
        int c = 0;
        while (c < c_end) {
            if (P.fresh[c]) { ++c; continue; }
            int e = c;
            while (e < c_end && !P.fresh[e] && e - c < 32 && P.cmax_valid[e] == P.cmax_valid[c]) ++e;
            const int nc = e - c;
            if (!P.cmax_valid[c]) {
                zj.push_back({P.cmax + c, (int)(nc * sizeof(unsigned long long))});
                const int nrb = (int)ceil_div(P.m, 4096);
                cj.push_back({P.X, P.ld, P.m, c, nrb, P.cmax});
                cc.push_back(nrb * nc);
            }
            const int ntile = (int)ceil_div(P.m, 128);
            sj.push_back({P.X, P.ld, P.m, P.nrc, P.n, c, nc, ntile, P.cmax, P.cexp, P.colstore});
            sc.push_back(ntile * (int)ceil_div(nc, 16));
            for (int k = c; k < e; ++k) { P.fresh[k] = 1; P.cmax_valid[k] = 0; }
            c = e;
        }
    };

    std::vector<SplitGramJob> gj, gj16;
    std::vector<int> gc, gc16;
    std::vector<GramJob> rj;
    std::vector<int> rc2;
    bool too_big = false;   // a Gram's partials would not fit the matrix's buffer
    // launch_gram_split's parameters for one matrix.
    auto gram = [&](SMat& M, int na, int b0, int nb, double* C, int ldc) {
        prepare(M, na > b0 + nb ? na : b0 + nb);
        Plan& P = M.P;
        GramParams gp{};
        gp.na = na; gp.nb = nb; gp.b0 = b0; gp.m = P.m;
        const int NB = nb <= 16 ? 16 : 32;   // as launch_gram_split
        gp.numMB = (int)ceil_div(na, TILE_M);
        gp.numNG = (int)ceil_div(nb, NB);
        const int mbn = gp.numMB * gp.numNG;
        gp.rc = S.num_sms / mbn > 0 ? S.num_sms / mbn : 1;
        gp.rows_per = round_up(ceil_div(P.m, gp.rc), (i64)ROW_ALIGN);
        gp.rc = (int)ceil_div(P.m, gp.rows_per);
        gp.nrc = (int)P.nrc;
        gp.cexp = P.cexp;
        gp.part = P.part;
        gp.err = nullptr;
        gp.a_once = gp.numNG == 1 ? 1 : 0;
        gp.alast = (int)round_up(na - (i64)(gp.numMB - 1) * TILE_M, 16);
        if ((i64)gp.rc * na * nb > P.part_doubles) too_big = true;
        SplitGramJob J;
        std::memset(&J, 0, sizeof(J));
        J.mapA = P.map_col_a;
        J.mapAlast = gp.alast < TILE_M ? P.map_col_a_part[gp.alast / 16 - 1] : P.map_col_a;
        J.mapB = NB == 16 ? P.map_col_b16 : P.map_col_b;
        J.p = gp;
        (NB == 16 ? gj16 : gj).push_back(J);
        (NB == 16 ? gc16 : gc).push_back(mbn * gp.rc);
        GramJob R{};
        R.na = na; R.nb = nb; R.nchunks = gp.rc; R.part = P.part; R.C = C; R.ldc = ldc;
        rj.push_back(R);
        rc2.push_back((int)ceil_div((i64)na * nb, 256));
    };
    auto flush_gram = [&]() {
        flush_prepare();
        push(kSGram, gj, gc);
        push(kSGram16, gj16, gc16);
        push(kSReduce, rj, rc2);
        gj.clear(); gc.clear(); gj16.clear(); gc16.clear(); rj.clear(); rc2.clear();
    };

    std::vector<SmallJob> smj;
    auto flush_small = [&]() {
        if (smj.empty()) return;
        std::vector<int> ones(smj.size(), 1);
        push(kSSmall, smj, ones);
        smj.clear();
    };
    auto pyth = [](const double* Om, int ldom, const double* A, int lda, int k, int nz, double* T, int step) {
        SmallSub X{};
        X.kind = kSmallPyth;
        X.p0 = Om; X.ld0 = ldom; X.p1 = A; X.ld1 = lda; X.a = k; X.b = nz; X.out = T; X.ldo = nz; X.step = step;
        return X;
    };
    auto scol = [](const double* G, int ldg, int mZ, int s, int nZ, const double* Yd, double* Scol) {
        SmallSub X{};
        X.kind = kSmallScol;
        X.p0 = G; X.ld0 = ldg; X.a = mZ; X.b = s; X.c = nZ; X.p1 = Yd; X.ld1 = s; X.out = Scol; X.ldo = mZ + s;
        return X;
    };
    auto rblock = [](int c0, int K, int ny, const double* A, int lda, const double* Bm, int ldb, const double* Sd,
                     const double* Yd) {
        SmallSub X{};
        X.kind = kSmallRblock;
        X.a = c0; X.b = K; X.c = ny; X.d = 0;
        X.p0 = A; X.ld0 = lda; X.p1 = Bm; X.ld1 = ldb; X.p2 = Sd; X.ld2 = ny; X.p3 = Yd; X.ld3 = ny;
        return X;
    };

    std::vector<ZeroJob> uz;
    std::vector<BbuildJob> bj;
    std::vector<int> bc;
    std::vector<BdigitJob> dj;
    std::vector<int> dc;
    std::vector<SplitUpdJob> uj, uj16;
    std::vector<int> ut, ut16;
    // finish_update for one matrix: kin digit columns in, nout (<= 32) columns out at
    // c0; as finish_update, 16-column tiles when nout <= 16 (blocks of s <= 8), each
    // width one batched launch.
    auto finish = [&](SMat& M, int kin, int c0, int nout) {
        Plan& P = M.P;
        const int NB = nout <= 16 ? 16 : 32;
        dj.push_back({P.bfull, (int)P.kpad, kin - nout, nout, NB, (int)P.kpad, P.bmax, P.fexp, P.bdig});
        dc.push_back((int)ceil_div(P.kpad, 256));
        uz.push_back({P.cmax + c0, (int)(nout * sizeof(unsigned long long))});
        UpdateParams up{};
        up.nrc = (int)P.nrc;
        up.m = P.m; up.kin = kin; up.nc = nout; up.c0 = c0; up.ld = P.ld; up.X = P.X; up.fexp = P.fexp;
        up.cmax = P.cmax; up.err = nullptr; up.tile_ctr = nullptr;
        up.kr_last = (int)round_up(kin - (i64)(ceil_div(kin, KCH) - 1) * KCH, 16);
        SplitUpdJob J;
        std::memset(&J, 0, sizeof(J));
        J.mapA = P.map_col_u;
        J.mapAlast = up.kr_last < KCH ? P.map_col_u_part[up.kr_last / 16 - 1] : P.map_col_u;
        J.mapB = NB == 16 ? P.map_bdig16 : P.map_bdig32;
        J.p = up;
        (NB == 16 ? uj16 : uj).push_back(J);
        (NB == 16 ? ut16 : ut).push_back((int)ceil_div(P.m, TILE_M));
        for (int c = c0; c < c0 + nout; ++c) { P.fresh[c] = 0; P.cmax_valid[c] = 1; }
    };
    // Engine::update (launch_update_split): X[:, c0:c0+nc] = (X_c - X[:, 0:K] S) T^{-1}, c0 == K.
    auto update = [&](SMat& M, int K, int c0, int nc, const double* Sm, int lds, const double* T, int ldt) {
        prepare(M, K + nc);
        Plan& P = M.P;
        uz.push_back({P.bmax, (int)(64 * sizeof(unsigned long long))});
        BbuildJob B{};
        B.fused = 0; B.S = Sm; B.lds = lds; B.T = T; B.ldt = ldt; B.K = K; B.nc = nc;
        B.cexp = P.cexp; B.Bp = P.bfull; B.ldb = (int)P.kpad; B.bmax = P.bmax;
        bj.push_back(B);
        bc.push_back((int)ceil_div(K + nc, 64));
        finish(M, K + nc, c0, nc);
    };
    // Engine::fused_update (launch_fused_update_split).
    auto fused = [&](SMat& M, int K, int nz, const double* G, int ldg, const double* Ty, const double* Sp,
                     const double* Ts) {
        const int s = M.s;
        prepare(M, K + s + nz);
        Plan& P = M.P;
        uz.push_back({P.bmax, (int)(128 * sizeof(unsigned long long))});
        BbuildJob B{};
        B.fused = 1; B.G = G; B.ldg = ldg; B.K = K; B.s = s; B.Ty = Ty; B.Sp = Sp; B.ldsp = K + s; B.Ts = Ts;
        B.nz = nz; B.cexp = P.cexp; B.Bp = P.bfull; B.ldb = (int)P.kpad; B.bmax = P.bmax;
        bj.push_back(B);
        bc.push_back((int)ceil_div(K + s + nz, 64));
        finish(M, K + s + nz, K, s + nz);
    };
    auto flush_update = [&]() {
        flush_prepare();
        if (uj.empty() && uj16.empty()) return;
        if (S.device) uz.push_back({S.dtile, (int)(2 * sizeof(int))});   // both launches' tile counters
        push_zero(uz);
        push(kSBbuild, bj, bc);
        push(kSBdigit, dj, dc);
        if (!uj.empty()) push(kSUpdate, uj, ut);
        if (!uj16.empty()) push(kSUpdate16, uj16, ut16);
        uz.clear(); bj.clear(); bc.clear(); dj.clear(); dc.clear(); uj.clear(); ut.clear(); uj16.clear(); ut16.clear();
    };

    // ---- TSQR of block 1 (the single-panel tree of launch_tsqr, per matrix) ----
    {
        constexpr int TR = 256;
        struct Lv { double* ptr; i64 rows, ld; };
        std::vector<std::vector<Lv>> lv;
        std::vector<double*> rroot;
        int Lmax = 0;
        for (int i : W.mats) {
            SMat& M = S.mats[i];
            std::vector<Lv> v;
            v.push_back({M.X, M.m, M.ld});
            double* cursor = M.tsqr;
            while (v.back().rows > TR) {
                const i64 tiles = ceil_div(v.back().rows, TR);
                double* next = cursor;
                cursor = cursor ? cursor + tiles * M.s * M.s : nullptr;
                v.push_back({next, tiles * M.s, tiles * M.s});
            }
            rroot.push_back(cursor);
            Lmax = std::max(Lmax, (int)v.size() - 1);
            lv.push_back(v);
        }
        const int B = (int)W.mats.size();
        for (int l = 0; l <= Lmax; ++l) {
            std::vector<TsqrTileJob> jobs;
            std::vector<int> counts;
            for (int k = 0; k < B; ++k) {
                const SMat& M = S.mats[W.mats[k]];
                const int L = (int)lv[k].size() - 1;
                if (l > L) continue;
                const Lv& v = lv[k][l];
                TsqrTileJob J;
                J.A = v.ptr; J.lda = v.ld; J.rows = v.rows; J.nc = M.s;
                if (l < L) {
                    const i64 tiles = ceil_div(v.rows, TR);
                    J.Rst = lv[k][l + 1].ptr; J.ldr = tiles * M.s;
                    counts.push_back((int)tiles);
                } else {
                    J.Rst = rroot[k]; J.ldr = M.s;
                    counts.push_back(1);
                }
                jobs.push_back(J);
            }
            push(kSTile, jobs, counts);
        }
        {
            std::vector<TsqrRootJob> jobs;
            std::vector<int> counts;
            for (int k = 0; k < B; ++k) {
                const SMat& M = S.mats[W.mats[k]];
                const Lv& v = lv[k].back();
                TsqrRootJob J;
                J.Q = v.ptr; J.ldq = v.ld; J.hq = (int)v.rows; J.nc = M.s;
                J.R = rroot[k]; J.ldr = M.s; J.Rout = M.R; J.ldro = M.ldR;
                jobs.push_back(J);
                counts.push_back(1);
            }
            push(kSRoot, jobs, counts);
        }
        for (int l = Lmax - 1; l >= 0; --l) {
            std::vector<TsqrApplyJob> jobs;
            std::vector<int> counts;
            for (int k = 0; k < B; ++k) {
                const SMat& M = S.mats[W.mats[k]];
                const int L = (int)lv[k].size() - 1;
                if (l >= L) continue;
                TsqrApplyJob J;
                J.Q = lv[k][l].ptr; J.ldq = lv[k][l].ld; J.rows = lv[k][l].rows; J.nc = M.s; J.TR = TR;
                J.P = lv[k][l + 1].ptr; J.ldp = lv[k][l + 1].ld;
                jobs.push_back(J);
                counts.push_back((int)ceil_div(J.rows, 128));
            }
            push(kSApply, jobs, counts);
        }
        for (int i : W.mats) {
            SMat& M = S.mats[i];
            for (int c = 0; c < M.s; ++c) { M.P.fresh[c] = 0; M.P.cmax_valid[c] = 0; }
        }
    }

    // ---- the schedule of run_lagged_fused (pyth = true), phase by phase ----
    const int B = (int)W.mats.size();
    std::vector<int> nZ(B), mZ(B), ldg(B);
    int pmax = 0;
    for (int k = 0; k < B; ++k) pmax = std::max(pmax, S.mats[W.mats[k]].p);
    // Phase 0: W = X_{1:2}^T X_2 (:111-114), Sdiag (:115-119), U_2 (:121-124).
    for (int k = 0; k < B; ++k) {
        SMat& M = S.mats[W.mats[k]];
        gram(M, 2 * M.s, M.s, M.s, M.G2, 2 * M.s);
    }
    flush_gram();
    for (int k = 0; k < B; ++k) {
        SMat& M = S.mats[W.mats[k]];
        SmallJob J{};
        J.status = M.status; J.R = M.R; J.ldR = M.ldR;
        J.sub[0] = pyth(M.G2 + M.s, 2 * M.s, M.G2, 2 * M.s, M.s, M.s, M.Sd, 1);
        J.nsub = 1;
        smj.push_back(J);
    }
    flush_small();
    for (int k = 0; k < B; ++k) {
        SMat& M = S.mats[W.mats[k]];
        update(M, M.s, M.s, M.s, M.G2, 2 * M.s, M.Sd, M.s);
    }
    flush_update();
    // Phase 1: the first synchronization of Q_2 (:127-147), then Q_2 and U_3.
    for (int k = 0; k < B; ++k) {
        SMat& M = S.mats[W.mats[k]];
        const int s = M.s;
        nZ[k] = M.n - s - s < s ? M.n - s - s : s;
        const int na = 2 * s + nZ[k], nb = s + nZ[k];
        gram(M, na, s, nb, M.G1, na);
        ldg[k] = na;
        mZ[k] = s;
    }
    flush_gram();
    for (int k = 0; k < B; ++k) {
        SMat& M = S.mats[W.mats[k]];
        const int s = M.s;
        SmallJob J{};
        J.status = M.status; J.R = M.R; J.ldR = M.ldR;
        J.sub[0] = pyth(M.G1 + s, ldg[k], M.G1, ldg[k], s, s, M.Yd, 1);
        J.sub[1] = rblock(s, s, s, M.G2, 2 * s, M.G1, ldg[k], M.Sd, M.Yd);
        J.nsub = 2;
        if (M.p > 1) {
            const int mScolN = mZ[k] + s;
            J.sub[2] = scol(M.G1, ldg[k], mZ[k], s, nZ[k], M.Yd, M.Scol);
            J.sub[3] = pyth(M.G1 + mScolN + (i64)s * ldg[k], ldg[k], M.Scol, mScolN, mScolN, nZ[k], M.Sd, 2);
            J.nsub = 4;
        }
        smj.push_back(J);
    }
    flush_small();
    for (int k = 0; k < B; ++k) {
        SMat& M = S.mats[W.mats[k]];
        const int s = M.s;
        if (M.p <= 1) update(M, s, s, s, M.G1, ldg[k], M.Yd, s);
        else fused(M, s, nZ[k], M.G1, ldg[k], M.Yd, M.Scol, M.Sd);
    }
    flush_update();
    // Phases 2 .. pmax: block step i = phase - 1 (:152-218).
    std::vector<int> nY(B), nZn(B);
    for (int ph = 2; ph <= pmax; ++ph) {
        const int i = ph - 1;
        for (int k = 0; k < B; ++k) {
            SMat& M = S.mats[W.mats[k]];
            if (i > M.p - 1) continue;
            const int s = M.s, n = M.n, mScol = mZ[k] + s;
            int na, nb;
            if (i < M.p - 1) {
                nZn[k] = n - (i + 1) * s - s < s ? n - (i + 1) * s - s : s;
                na = mScol + s + nZn[k];
                nb = s + nZn[k];
                nY[k] = s;
            } else {
                nZn[k] = nZ[k];
                na = mScol + nZ[k];
                nb = nZ[k];
                nY[k] = nZ[k];
            }
            gram(M, na, mScol, nb, M.G1, na);
            ldg[k] = na;
        }
        flush_gram();
        for (int k = 0; k < B; ++k) {
            SMat& M = S.mats[W.mats[k]];
            if (i > M.p - 1) continue;
            const int s = M.s, mScol = mZ[k] + s;
            SmallJob J{};
            J.status = M.status; J.R = M.R; J.ldR = M.ldR;
            J.sub[0] = pyth(M.G1 + mScol, ldg[k], M.G1, ldg[k], mScol, nY[k], M.Yd, i + 1);
            J.sub[1] = rblock(mScol, mScol, nY[k], M.Scol, mScol, M.G1, ldg[k], M.Sd, M.Yd);
            J.nsub = 2;
            if (i < M.p - 1) {
                const int mZn = mZ[k] + s, mScolN = mZn + s;
                J.sub[2] = scol(M.G1, ldg[k], mZn, s, nZn[k], M.Yd, M.Scol);
                J.sub[3] = pyth(M.G1 + mScolN + (i64)s * ldg[k], ldg[k], M.Scol, mScolN, mScolN, nZn[k], M.Sd, i + 2);
                J.nsub = 4;
            }
            smj.push_back(J);
        }
        flush_small();
        for (int k = 0; k < B; ++k) {
            SMat& M = S.mats[W.mats[k]];
            if (i > M.p - 1) continue;
            const int s = M.s, mScol = mZ[k] + s;
            if (i < M.p - 1) fused(M, mScol, nZn[k], M.G1, ldg[k], M.Yd, M.Scol, M.Sd);
            else update(M, mScol, mScol, nY[k], M.G1, ldg[k], M.Yd, nY[k]);
            mZ[k] += s;
            nZ[k] = nZn[k];
        }
        flush_update();
    }
    return too_big ? (int)cudaErrorInvalidValue : 0;
}

int enqueue_wave(SplitStaged& S, SWave& W, cudaStream_t st) {
    char* jb = static_cast<char*>(W.blob_dev);
    const long long k0 = g_launch_count;
    const int KD = S.kd;
    GramParams g0{};
    g0.err = S.derr;
    UpdateParams u0{};
    u0.err = S.derr;
    u0.tile_ctr = S.dtile;
    CUtensorMap none;
    std::memset(&none, 0, sizeof(none));
    for (const SLaunch& L : W.launches) {
        const int* pre = reinterpret_cast<const int*>(jb + L.prefix_off);
        const unsigned items = (unsigned)L.items;
        int rc = 0;
        switch (L.kind) {
            case kSZeroBuf: rc = zero_async(S.buf, (size_t)L.bytes, st); break;
            case kSZero:
                zero_list<<<items, 256, 0, st>>>(reinterpret_cast<const ZeroJob*>(jb + L.job_off));
                ++g_launch_count;
                break;
            case kSColmax:
                colmax_batched<<<items, 256, 0, st>>>(reinterpret_cast<const ColmaxJob*>(jb + L.job_off), pre, L.njobs);
                ++g_launch_count;
                break;
            case kSSlice:
                if (KD == 6)
                    slice_batched<6><<<items, 128, 0, st>>>(reinterpret_cast<const SliceJob*>(jb + L.job_off), pre,
                                                            L.njobs);
                else
                    slice_batched<7><<<items, 128, 0, st>>>(reinterpret_cast<const SliceJob*>(jb + L.job_off), pre,
                                                            L.njobs);
                ++g_launch_count;
                break;
            case kSGram:
            case kSGram16: {
                const auto* J = reinterpret_cast<const SplitGramJob*>(jb + L.job_off);
                const int ka = gram_a_planes(KD);
#define BCGS_GRAMB(NBT, KDT, KAT)                                                                              \
    gram_tc_kernel<NBT, KDT, KAT, true><<<items, NTHREADS, SmemLayout<NBT, KDT>::BYTES, st>>>(none, none, none, \
                                                                                            g0, J, pre, L.njobs)
                if (L.kind == kSGram16) {
                    if (KD == 6) BCGS_GRAMB(16, 6, 6); else if (ka == 6) BCGS_GRAMB(16, 7, 6); else BCGS_GRAMB(16, 7, 7);
                } else {
                    if (KD == 6) BCGS_GRAMB(32, 6, 6); else if (ka == 6) BCGS_GRAMB(32, 7, 6); else BCGS_GRAMB(32, 7, 7);
                }
#undef BCGS_GRAMB
                ++g_launch_count;
                break;
            }
            case kSReduce:
                rc = launch_gram_reduce_batched(reinterpret_cast<const GramJob*>(jb + L.job_off), pre, L.njobs,
                                                L.items, st);
                break;
            case kSSmall:
                rc = launch_small_batched(reinterpret_cast<const SmallJob*>(jb + L.job_off), L.njobs, st);
                break;
            case kSBbuild:
                bbuild_batched<<<items, 256, kBbuildSmem, st>>>(reinterpret_cast<const BbuildJob*>(jb + L.job_off), pre,
                                                               L.njobs);
                ++g_launch_count;
                break;
            case kSBdigit:
                if (KD == 6)
                    bdigit_batched<6><<<items, 256, 0, st>>>(reinterpret_cast<const BdigitJob*>(jb + L.job_off), pre,
                                                             L.njobs);
                else
                    bdigit_batched<7><<<items, 256, 0, st>>>(reinterpret_cast<const BdigitJob*>(jb + L.job_off), pre,
                                                             L.njobs);
                ++g_launch_count;
                break;
            case kSUpdate: {
                const auto* J = reinterpret_cast<const SplitUpdJob*>(jb + L.job_off);
                const unsigned grid = items < (unsigned)S.num_sms ? items : (unsigned)S.num_sms;
                if (KD == 6)
                    update_tc_kernel<32, 6, true><<<grid, UTHREADS, SmemLayout<32, 6>::BYTES, st>>>(none, none, none, u0,
                                                                                                   J, pre, L.njobs);
                else
                    update_tc_kernel<32, 7, true><<<grid, UTHREADS, SmemLayout<32, 7>::BYTES, st>>>(none, none, none, u0,
                                                                                                   J, pre, L.njobs);
                ++g_launch_count;
                break;
            }
            case kSUpdate16: {   // its own tile counter: the word after the 32-column launch's
                const auto* J = reinterpret_cast<const SplitUpdJob*>(jb + L.job_off);
                const unsigned grid = items < (unsigned)S.num_sms ? items : (unsigned)S.num_sms;
                UpdateParams u16 = u0;
                u16.tile_ctr = S.dtile + 1;
                if (KD == 6)
                    update_tc_kernel<16, 6, true><<<grid, UTHREADS, SmemLayout<16, 6>::BYTES, st>>>(none, none, none, u16,
                                                                                                   J, pre, L.njobs);
                else
                    update_tc_kernel<16, 7, true><<<grid, UTHREADS, SmemLayout<16, 7>::BYTES, st>>>(none, none, none, u16,
                                                                                                   J, pre, L.njobs);
                ++g_launch_count;
                break;
            }
            case kSTile:
                rc = launch_tsqr_tile_batched(reinterpret_cast<const TsqrTileJob*>(jb + L.job_off), pre, L.njobs,
                                              L.items, 16, st);
                break;
            case kSRoot:
                rc = launch_tsqr_root_batched(reinterpret_cast<const TsqrRootJob*>(jb + L.job_off), L.njobs, st);
                break;
            case kSApply:
                rc = launch_tsqr_apply_batched(reinterpret_cast<const TsqrApplyJob*>(jb + L.job_off), pre, L.njobs,
                                               L.items, 16, st);
                break;
            default: rc = (int)cudaErrorInvalidValue;
        }
        if (!rc) rc = (int)cudaGetLastError();
        if (rc) return rc;
    }
    W.kernels = g_launch_count - k0;
    return 0;
}

void free_staged(SplitStaged* S) {
    if (!S) return;
    for (SWave& W : S->waves) {
        if (W.exec) cudaGraphExecDestroy(W.exec);
        if (W.graph) cudaGraphDestroy(W.graph);
        if (W.blob_dev) cudaFree(W.blob_dev);
    }
    if (S->buf) cudaFree(S->buf);
    if (S->derr) cudaFree(S->derr);
    if (S->own) cudaStreamDestroy(S->own);
    delete S;
}

// Matrices into waves, in batch order: a wave takes matrices while their regions
// fit in `budget` bytes (at least one matrix per wave).
void assign_waves(SplitStaged& S, long long budget) {
    S.waves.clear();
    SWave cur;
    size_t used = 0;
    for (int i = 0; i < S.count; ++i) {
        SMat& M = S.mats[i];
        const size_t b = (smat_layout(M, S.num_sms, nullptr) + 4095) & ~(size_t)4095;
        if (!cur.mats.empty() && budget > 0 && (long long)(used + b) > budget) {
            S.waves.push_back(std::move(cur));
            cur = SWave();
            used = 0;
        }
        cur.mats.push_back(i);
        used += b;
    }
    if (!cur.mats.empty()) S.waves.push_back(std::move(cur));
}

int fill_smats(SplitStaged& S, int count, const int* m, const int* n, const int* s, double* const* dX,
               const long long* ldX, double* const* dR, const int* ldR, int* dstatus) {
    S.count = count;
    S.mats.resize(count);
    for (int b = 0; b < count; ++b) {
        SMat& M = S.mats[b];
        M.b = b; M.m = m[b]; M.n = n[b]; M.s = s[b];
        M.ld = ldX ? ldX[b] : m[b];
        M.X = dX ? dX[b] : nullptr;
        M.R = dR ? dR[b] : nullptr;
        M.ldR = ldR ? ldR[b] : n[b];
        M.status = dstatus ? dstatus + 8 * (i64)b : nullptr;
        if (M.s < 1 || M.s > 16 || M.n < 2 * M.s || M.m < M.n || M.ld < M.m || M.ldR < M.n || M.m < TILE_M) return 2;
        M.p = (M.n - M.s + M.s - 1) / M.s;
    }
    return 0;
}

}  // namespace

bool split_staged_supported(int variant, int count, const int* s) {
    if (variant != ORTH_GB300_BCGSI2P1S) return false;
    for (int b = 0; b < count; ++b)
        if (s[b] < 1 || s[b] > 16) return false;
    return true;
}

int split_staged_create(int count, const int* m, const int* n, const int* s, double* const* dX,
                        const long long* ldX, double* const* dR, const int* ldR, int kd, int* dstatus,
                        long long budget, cudaStream_t st, SplitStaged** out) {
    *out = nullptr;
    SplitStaged* S = new SplitStaged();
    S->kd = kd;
    S->dstatus = dstatus;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&S->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        free_staged(S);
        return 3;
    }
    int rc = fill_smats(*S, count, m, n, s, dX, ldX, dR, ldR, dstatus);
    if (rc) { free_staged(S); return rc; }
    // Shared-memory limits of the batched kernels on this device.
    rc = set_smem(gram_tc_kernel<32, 6, 6, true>, SmemLayout<32, 6>::BYTES);
    if (!rc) rc = set_smem(gram_tc_kernel<32, 7, 7, true>, SmemLayout<32, 7>::BYTES);
    if (!rc) rc = set_smem(gram_tc_kernel<32, 7, 6, true>, SmemLayout<32, 7>::BYTES);
    if (!rc) rc = set_smem(gram_tc_kernel<16, 6, 6, true>, SmemLayout<16, 6>::BYTES);
    if (!rc) rc = set_smem(gram_tc_kernel<16, 7, 7, true>, SmemLayout<16, 7>::BYTES);
    if (!rc) rc = set_smem(gram_tc_kernel<16, 7, 6, true>, SmemLayout<16, 7>::BYTES);
    if (!rc) rc = set_smem(update_tc_kernel<32, 6, true>, SmemLayout<32, 6>::BYTES);
    if (!rc) rc = set_smem(update_tc_kernel<32, 7, true>, SmemLayout<32, 7>::BYTES);
    if (!rc) rc = set_smem(update_tc_kernel<16, 6, true>, SmemLayout<16, 6>::BYTES);
    if (!rc) rc = set_smem(update_tc_kernel<16, 7, true>, SmemLayout<16, 7>::BYTES);
    if (!rc) rc = set_smem(bbuild_batched, (int)kBbuildSmem);
    if (!rc) rc = tsqr_tile_batched_prepare();
    if (rc) { free_staged(S); return 3; }
    if (budget < 0) {
        const char* e = getenv("ORTH_GB300_SPLIT_WAVE_BYTES");
        if (e && atoll(e) > 0) budget = atoll(e);
    }
    if (budget < 0) {
        size_t fb = 0, tb = 0;
        if (cudaMemGetInfo(&fb, &tb) != cudaSuccess) { free_staged(S); return 3; }
        budget = (long long)((double)fb * 0.85) - (256LL << 20);
        if (budget < (256LL << 20)) budget = 256LL << 20;
    }
    assign_waves(*S, budget);
    size_t need = 0;
    for (SWave& W : S->waves) {
        size_t u = 0;
        for (int i : W.mats) u += (smat_layout(S->mats[i], S->num_sms, nullptr) + 4095) & ~(size_t)4095;
        need = std::max(need, u);
    }
    S->buf_bytes = need;
    if (cudaMalloc(&S->buf, need) != cudaSuccess || cudaMalloc(&S->derr, 64) != cudaSuccess ||
        cudaMemset(S->derr, 0, 64) != cudaSuccess ||
        cudaStreamCreateWithFlags(&S->own, cudaStreamNonBlocking) != cudaSuccess) {
        (void)cudaGetLastError();
        free_staged(S);
        return 3;
    }
    S->dtile = S->derr + 1;
    for (SWave& W : S->waves) {
        rc = plan_wave(*S, W);
        if (rc) { free_staged(S); return 3; }
        if (cudaMalloc(&W.blob_dev, W.blob.bytes.size() + 128) != cudaSuccess ||
            cudaMemcpy(W.blob_dev, W.blob.bytes.data(), W.blob.bytes.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
            free_staged(S);
            return 3;
        }
    }
    // Capture each wave; the first also clears the status words and the error
    // word, the last copies the error word into every matrix's status.
    if (cudaStreamSynchronize(st) != cudaSuccess) { free_staged(S); return 3; }
    for (size_t w = 0; w < S->waves.size(); ++w) {
        SWave& W = S->waves[w];
        if (cudaStreamBeginCapture(S->own, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { free_staged(S); return 3; }
        rc = 0;
        if (w == 0) {
            rc = zero_async(S->dstatus, (size_t)S->count * 8 * sizeof(int), S->own);
            if (!rc) rc = zero_async(S->derr, sizeof(int), S->own);
        }
        if (!rc) rc = enqueue_wave(*S, W, S->own);
        if (!rc && w + 1 == S->waves.size()) {
            spread_error<<<(unsigned)ceil_div(S->count, 256), 256, 0, S->own>>>(S->derr, S->dstatus, S->count);
            ++g_launch_count;
            rc = (int)cudaGetLastError();
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(S->own, &g);
        if (rc || ce != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            free_staged(S);
            return 3;
        }
        W.graph = g;
        if (cudaGraphInstantiate(&W.exec, g, 0) != cudaSuccess) { free_staged(S); return 3; }
        size_t nodes = 0;
        cudaGraphGetNodes(g, nullptr, &nodes);
        S->nodes += (int)nodes;
        S->kernels += W.kernels + (w == 0 ? 2 : 0) + (w + 1 == S->waves.size() ? 1 : 0);
    }
    *out = S;
    return 0;
}

int split_staged_run(SplitStaged* S, cudaStream_t st) {
    if (!S) return 2;
    for (SWave& W : S->waves)
        if (cudaGraphLaunch(W.exec, st) != cudaSuccess) return 3;
    g_launch_count += S->kernels;
    return 0;
}

void split_staged_destroy(SplitStaged* S) { free_staged(S); }

void split_staged_info(const SplitStaged* S, long long* kernels, long long* bytes, int* nodes, int* waves) {
    if (!S) return;
    if (kernels) *kernels = S->kernels;
    if (bytes) *bytes = (long long)S->buf_bytes;
    if (nodes) *nodes = S->nodes;
    if (waves) *waves = (int)S->waves.size();
}

int split_staged_dry_run(int count, const int* m, const int* n, const int* s, long long budget, int* waves,
                         long long* kernels, long long* bytes) {
    SplitStaged S;
    S.device = false;
    S.num_sms = kNumSMsDefault;
    int rc = fill_smats(S, count, m, n, s, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (rc) return rc;
    assign_waves(S, budget);
    long long k = 4;   // the status and error clears, the error spread, one buffer clear per wave below
    size_t need = 0;
    for (SWave& W : S.waves) {
        if (plan_wave(S, W)) return 2;
        k += (long long)W.launches.size() + 1;
        need = std::max(need, W.used);
    }
    k -= 1;
    if (waves) *waves = (int)S.waves.size();
    if (kernels) *kernels = k;
    if (bytes) *bytes = (long long)need;
    return 0;
}

}  // namespace bcgs
