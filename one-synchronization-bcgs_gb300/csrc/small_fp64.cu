// Small FP64 block kernels of the BCGS step (one CTA each, s <= 64).
//
// These run between the tall passes on the reduced Gram blocks and replace the
// reference's small dgemm/dtrsm/dpotrf calls on s x s and K x s matrices:
//   pyth_chol : T = chol(Om - A^T A), upper       (SRC/orth.c:160-171, 200-204, ...)
//   scol      : S = Q_{1:k-1}^T X_k reconstructed  (SRC/orth.c:155-159, 310-314, 641-645)
//   rblock    : R column block assembly            (SRC/orth.c:211-215, 356-360, ...)
// Work here is O(K s^2) per step, negligible next to the tall passes, but it
// sits on the critical path, so every step keeps it on the device: no host
// round trip between the synchronizations.
#include "batched.h"
#include "common.cuh"
#include "kernels.h"

namespace bcgs {

namespace {
constexpr int SM_THREADS = 256;
constexpr int SMAX = 64;
}  // namespace

// Cholesky of the upper triangle of the nz x nz matrix in shared memory `a`
// (column-major, ld SMAX), the unblocked row-oriented algorithm of LAPACK's
// dpotf2 ('U'): for j = 0..nz-1,
//   ajj = a_jj - sum_{i<j} a_ij^2; if ajj <= 0 stop with info = j+1 and a_jj = ajj;
//   a_jj = sqrt(ajj); a_jc = (a_jc - sum_{i<j} a_ij a_ic) / a_jj for c > j.
// On breakdown the partial factor is left in place, as dpotrf leaves it.
__device__ int chol_upper_shared(double* a, int nz) {
    __shared__ int s_info;
    __shared__ double s_ajj;
    if (threadIdx.x == 0) s_info = 0;
    __syncthreads();
    for (int j = 0; j < nz; ++j) {
        if (threadIdx.x == 0) {
            double ajj = a[j + j * SMAX];
            for (int i = 0; i < j; ++i) ajj -= a[i + j * SMAX] * a[i + j * SMAX];
            if (ajj <= 0.0) {
                a[j + j * SMAX] = ajj;
                s_info = j + 1;
            } else {
                ajj = sqrt(ajj);
                a[j + j * SMAX] = ajj;
            }
            s_ajj = ajj;
        }
        __syncthreads();
        if (s_info != 0) break;
        const double rajj = 1.0 / s_ajj;
        for (int c = j + 1 + (int)threadIdx.x; c < nz; c += blockDim.x) {
            double v = a[j + c * SMAX];
            for (int i = 0; i < j; ++i) v -= a[i + j * SMAX] * a[i + c * SMAX];
            a[j + c * SMAX] = v * rajj;
        }
        __syncthreads();
    }
    __syncthreads();
    return s_info;
}

// T(nz x nz, ld ldt) = chol_upper(Om(nz x nz, ld ldom) - A(k x nz, ld lda)^T A).
// Only the upper triangle of Om is read; T's strictly lower part is zeroed
// (dlaset 'L' + dlacpy 'U' + dpotrf 'U'). A may be null when k == 0.
// Body shared by the single and batched kernels; `a` is SMAX*SMAX doubles of shared
// memory. Starts and ends with a CTA barrier, so the caller may reuse `a`.
__device__ void pyth_chol_body(const double* __restrict__ Om, int ldom, const double* __restrict__ A, int lda,
                               int k, int nz, double* __restrict__ T, int ldt, int* __restrict__ status, int step,
                               double* __restrict__ a) {
    __syncthreads();
    for (int e = threadIdx.x; e < nz * nz; e += blockDim.x) {
        int i = e % nz, j = e / nz;
        double v = 0.0;
        if (i <= j) {
            v = Om[i + (i64)j * ldom];
            for (int l = 0; l < k; ++l) v -= A[l + (i64)i * lda] * A[l + (i64)j * lda];
        }
        a[i + j * SMAX] = v;
    }
    __syncthreads();
    int info = chol_upper_shared(a, nz);
    for (int e = threadIdx.x; e < nz * nz; e += blockDim.x) {
        int i = e % nz, j = e / nz;
        T[i + (i64)j * ldt] = (i <= j) ? a[i + j * SMAX] : 0.0;
    }
    if (threadIdx.x == 0 && info != 0 && status != nullptr && status[0] == 0) {
        status[0] = step;
        status[1] = info;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(SM_THREADS)
pyth_chol_kernel(const double* __restrict__ Om, int ldom, const double* __restrict__ A, int lda,
                 int k, int nz, double* __restrict__ T, int ldt, int* __restrict__ status, int step) {
    __shared__ double a[SMAX * SMAX];
    pyth_chol_body(Om, ldom, A, lda, k, nz, T, ldt, status, step, a);
}

// Scol(mScol x nZ, ld ldsc), mScol = mZ + s, from the last reduced Gram G (ld ldg):
//   Scol = G[0:mScol, s:s+nZ]
//   Scol[mZ:mScol] -= G[0:mZ, 0:s]^T G[0:mZ, s:s+nZ]
//   Scol[mZ:mScol]  = Ydiag^{-T} Scol[mZ:mScol]       (dtrsm 'L','U','T','N')
// Body shared by the single and batched kernels; dsm is SMAX*(nZ+s) doubles.
__device__ void scol_body(const double* __restrict__ G, int ldg, int mZ, int s, int nZ,
                          const double* __restrict__ Yd, int ldy, double* __restrict__ Scol, int ldsc,
                          double* __restrict__ dsm) {
    __syncthreads();
    double* b = dsm;               // s x nZ, ld SMAX (only s rows used)
    double* y = dsm + SMAX * nZ;   // s x s, ld SMAX
    for (int e = threadIdx.x; e < mZ * nZ; e += blockDim.x) {
        int i = e % mZ, j = e / mZ;
        Scol[i + (i64)j * ldsc] = G[i + (i64)(s + j) * ldg];
    }
    for (int e = threadIdx.x; e < s * nZ; e += blockDim.x) {
        int i = e % s, j = e / s;
        double v = G[(mZ + i) + (i64)(s + j) * ldg];
        for (int l = 0; l < mZ; ++l) v -= G[l + (i64)i * ldg] * G[l + (i64)(s + j) * ldg];
        b[i + j * SMAX] = v;
    }
    for (int e = threadIdx.x; e < s * s; e += blockDim.x) {
        int i = e % s, j = e / s;
        y[i + j * SMAX] = Yd[i + (i64)j * ldy];
    }
    __syncthreads();
    // Forward substitution with Yd^T (lower): z_i = (b_i - sum_{l<i} Yd_li z_l) / Yd_ii,
    // one right-hand side column per thread.
    for (int j = threadIdx.x; j < nZ; j += blockDim.x) {
        for (int i = 0; i < s; ++i) {
            double v = b[i + j * SMAX];
            for (int l = 0; l < i; ++l) v -= y[l + i * SMAX] * b[l + j * SMAX];
            b[i + j * SMAX] = v / y[i + i * SMAX];
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < s * nZ; e += blockDim.x) {
        int i = e % s, j = e / s;
        Scol[(mZ + i) + (i64)j * ldsc] = b[i + j * SMAX];
    }
    __syncthreads();
}

__global__ void __launch_bounds__(SM_THREADS)
scol_kernel(const double* __restrict__ G, int ldg, int mZ, int s, int nZ,
            const double* __restrict__ Yd, int ldy, double* __restrict__ Scol, int ldsc) {
    extern __shared__ double dsm[];
    scol_body(G, ldg, mZ, s, nZ, Yd, ldy, Scol, ldsc, dsm);
}

// R column block at columns [c0, c0+ny):
//   mode 0: R[0:K, c0:] = A + B Sd ;  R[c0:c0+ny, c0:] = Yd Sd      (P1s, PIPI, BCGSI+, P2s)
//   mode 1: R[0:K, c0:] = A + B    ;  upper(R[c0:c0+ny, c0:]) = upper(Yd)   (bcgsi21s)
// A, B are K x ny (ld lda, ldb); Sd, Yd upper ny x ny.
// Body shared by the single and batched kernels; sd is SMAX*SMAX doubles.
__device__ void rblock_body(double* __restrict__ R, int ldR, int c0, int K, int ny,
                            const double* __restrict__ A, int lda, const double* __restrict__ B, int ldb,
                            const double* __restrict__ Sd, int ldsd, const double* __restrict__ Yd, int ldyd,
                            int mode, double* __restrict__ sd) {
    __syncthreads();
    if (mode == 0) {
        for (int e = threadIdx.x; e < ny * ny; e += blockDim.x) {
            int i = e % ny, j = e / ny;
            sd[i + j * SMAX] = (i <= j) ? Sd[i + (i64)j * ldsd] : 0.0;
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < K * ny; e += blockDim.x) {
        int i = e % K, j = e / K;
        double v = A[i + (i64)j * lda];
        if (mode == 0) {
            double t = 0.0;
            for (int l = 0; l <= j; ++l) t += B[i + (i64)l * ldb] * sd[l + j * SMAX];
            v += t;
        } else {
            v += B[i + (i64)j * ldb];
        }
        R[i + (i64)(c0 + j) * ldR] = v;
    }
    for (int e = threadIdx.x; e < ny * ny; e += blockDim.x) {
        int i = e % ny, j = e / ny;
        double* dst = R + (c0 + i) + (i64)(c0 + j) * ldR;
        if (mode == 0) {
            double t = 0.0;
            if (i <= j)
                for (int l = i; l <= j; ++l) t += Yd[i + (i64)l * ldyd] * sd[l + j * SMAX];
            *dst = t;
        } else if (i <= j) {
            *dst = Yd[i + (i64)j * ldyd];
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(SM_THREADS)
rblock_kernel(double* __restrict__ R, int ldR, int c0, int K, int ny,
              const double* __restrict__ A, int lda, const double* __restrict__ B, int ldb,
              const double* __restrict__ Sd, int ldsd, const double* __restrict__ Yd, int ldyd,
              int mode) {
    __shared__ double sd[SMAX * SMAX];
    rblock_body(R, ldR, c0, K, ny, A, lda, B, ldb, Sd, ldsd, Yd, ldyd, mode, sd);
}

int launch_pyth_chol(const double* Om, int ldom, const double* A, int lda, int k, int nz,
                     double* T, int ldt, int* status, int step, cudaStream_t st) {
    if (nz <= 0) return 0;
    if (nz > SMAX) return (int)cudaErrorInvalidValue;
    pyth_chol_kernel<<<1, SM_THREADS, 0, st>>>(Om, ldom, A, lda, k, nz, T, ldt, status, step);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

int launch_scol(const double* G, int ldg, int mZ, int s, int nZ, const double* Yd, int ldy,
                double* Scol, int ldsc, cudaStream_t st) {
    if (nZ <= 0) return 0;
    if (s > SMAX || nZ > SMAX) return (int)cudaErrorInvalidValue;
    const size_t smem = (size_t)SMAX * (nZ + s) * sizeof(double);
    const int attr_rc = smem_attr((const void*)scol_kernel, (int)(SMAX * 2 * SMAX * sizeof(double)));
    if (attr_rc) return attr_rc;
    scol_kernel<<<1, SM_THREADS, smem, st>>>(G, ldg, mZ, s, nZ, Yd, ldy, Scol, ldsc);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

int launch_rblock(double* R, int ldR, int c0, int K, int ny, const double* A, int lda,
                  const double* B, int ldb, const double* Sd, int ldsd, const double* Yd,
                  int ldyd, int mode, cudaStream_t st) {
    if (ny <= 0) return 0;
    if (ny > SMAX) return (int)cudaErrorInvalidValue;
    rblock_kernel<<<1, SM_THREADS, 0, st>>>(R, ldR, c0, K, ny, A, lda, B, ldb, Sd, ldsd, Yd,
                                            ldyd, mode);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

// Batched form: one CTA per matrix runs that matrix's small operations of one stage
// in order (each with the single-matrix body, so the arithmetic is the same).
__global__ void __launch_bounds__(SM_THREADS)
small_batched(const SmallJob* __restrict__ jobs) {
    __shared__ double sm[SMAX * SMAX];
    const SmallJob& J = jobs[blockIdx.x];
    for (int q = 0; q < J.nsub; ++q) {
        const SmallSub& S = J.sub[q];
        if (S.kind == kSmallPyth)
            pyth_chol_body(S.p0, S.ld0, S.p1, S.ld1, S.a, S.b, S.out, S.ldo, J.status, S.step, sm);
        else if (S.kind == kSmallScol)
            scol_body(S.p0, S.ld0, S.a, S.b, S.c, S.p1, S.ld1, S.out, S.ldo, sm);
        else if (S.kind == kSmallRblock)
            rblock_body(J.R, J.ldR, S.a, S.b, S.c, S.p0, S.ld0, S.p1, S.ld1, S.p2, S.ld2, S.p3, S.ld3, S.d, sm);
    }
}

int launch_small_batched(const SmallJob* jobs, int njobs, cudaStream_t st) {
    if (njobs <= 0) return 0;
    small_batched<<<(unsigned)njobs, SM_THREADS, 0, st>>>(jobs);
    g_launch_count += 1;
    return (int)cudaGetLastError();
}

}  // namespace bcgs
