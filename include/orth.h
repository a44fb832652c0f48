/*
 * Drop-in C ABI of the reorthogonalized BCGS hot path for one GB300.
 *
 * The five entry points keep the reference's names, argument meanings, return
 * codes and buffer conventions (reference include/orth.h:8-17, implemented in
 * SRC/orth.c:48,224,369,464,550). Each one replaces the same-named function:
 *
 *   bcgsi2P1s  BCGSI+P-1S, one synchronization per block step (SRC/orth.c:48-222)
 *   bcgsi21s   BCGSI+A-1S, one synchronization per block step (SRC/orth.c:224-367)
 *   bcgspipi2  BCGS-PIPI+, two synchronizations per step       (SRC/orth.c:369-462)
 *   bcgsi2     BCGSI+ (BCGS2) with TSQR intra-orthogonalization  (SRC/orth.c:464-548)
 *   bcgsi2P2s  BCGSI+P-2S, TSQR first pass + one synchronization (SRC/orth.c:550-697)
 *
 * Arguments (column-major FP64, as in the reference; host memory as in the
 * reference, or device/managed memory, detected with cudaPointerGetAttributes):
 *   m       rows of X. With one GPU there is one rank, so Xsub holds all m rows.
 *   n, s    columns of X and the block width; n >= 2s, 1 <= s <= 64. The last
 *           block may be ragged (n - s not a multiple of s).
 *   Xsub    m x n, leading dimension ldXsub >= m; overwritten with Q. In host
 *           memory it is streamed to the GPU and back in column chunks while
 *           the QR runs; in device memory the QR runs on it in place.
 *   R       n x n, leading dimension ldR >= n; the upper block triangle is
 *           written, the rest is left untouched (host or device memory).
 *   work    not accessed (the GPU keeps its own workspace); lwork is checked
 *           with the reference's rule: >= 5ns + 9s^2 + m*n (m*s for bcgsi2),
 *           evaluated in 64 bits and capped at INT_MAX.
 *
 * Return codes: 0 success; 1 lwork too small (message on stdout, as the
 * reference prints); 2 invalid arguments; 3 CUDA failure. A Cholesky breakdown
 * of a Pythagorean-shifted Gram block does not change the return code (the
 * reference ignores dpotrf's info too); it is reported by
 * orth_gb300_last_status() in orth_gb300.h. Every call returns after its
 * results are in Xsub and R, as the reference's does.
 */
#ifndef ORTH_H
#define ORTH_H

#ifdef __cplusplus
extern "C" {
#endif
int bcgsi2P1s(int m, int n, int s, double *Xsub, int ldXsub, double *R,
        int ldR, double *work, int lwork);
int bcgsi21s(int m, int n, int s, double *Xsub, int ldXsub, double *R,
        int ldR, double *work, int lwork);
int bcgspipi2(int m, int n, int s, double *Xsub, int ldXsub, double *R,
        int ldR, double *work, int lwork);
int bcgsi2(int m, int n, int s, double *Xsub, int ldXsub, double *R,
        int ldR, double *work, int lwork);
int bcgsi2P2s(int m, int n, int s, double *Xsub, int ldXsub, double *R,
        int ldR, double *work, int lwork);
#ifdef __cplusplus
}
#endif

#endif
