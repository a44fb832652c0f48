"""CPU restatement of the reference's five reorthogonalized BCGS variants.

TEST INFRASTRUCTURE ONLY. This module is the oracle: tests, ``smoke()`` and the
``cpu_baseline`` leg of ``bench.py`` use it to check and to time against. The
product path (the CUDA library) never imports it.

Each function follows the reference's SRC/orth.c step by step, with the same
BLAS/LAPACK operations in the same order (scipy's LP64 OpenBLAS: dgemm, dtrsm,
dpotrf, dgeqrf, dorgqr), on one rank. A single-rank ``MPI_Allreduce`` is a copy,
so every reduction in the reference is the local Gram itself.

Conventions (mirroring ``include/orth.h`` of the reference):
  * ``X`` is an m x ncols float64 array in Fortran order, ncols >= n. Columns
    ``[0, n)`` are overwritten with Q. Callers should give at least ``n + s``
    columns when ``n < 3s`` because the reference's bcgsi2P1s reads ``s``
    columns of the third block even when fewer exist (SRC/orth.c:129-131).
  * ``R`` is an n x n float64 Fortran-order array; the upper block triangle is
    written, as in the reference.
  * The return value is ``info``: 0, or the 1-based step index of the first
    Cholesky (dpotrf) breakdown. The reference ignores dpotrf's info
    (SRC/orth.c:119,137,171,204,...) and carries on with the partial factor;
    this restatement carries on the same way and only records the step.

Intra-orthogonalization: the reference calls Trilinos TSQR ``factorExplicit``
(SRC/orth.c:14-46 and its call sites). Trilinos is not part of the reference;
its published contract is an explicit thin QR of the panel, restated here as
LAPACK Householder QR (dgeqrf + dorgqr). The sign of diag(R) is not forced, as
in the reference, so Q and R are compared up to column signs.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg.blas as _blas
import scipy.linalg.lapack as _lapack

__all__ = [
    "bcgsi2P1s", "bcgsi21s", "bcgspipi2", "bcgsi2", "bcgsi2P2s", "VARIANTS",
    "tsqr_explicit", "cholqr2_explicit", "loo_fro", "loo_2", "residual_fro", "rel_residual",
    "run_variant",
]


# --------------------------------------------------------------------------
# BLAS/LAPACK helpers: thin wrappers that keep the reference's in-place style.
# --------------------------------------------------------------------------
def _gram(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """dgemm('T','N'): A^T B as a new Fortran array."""
    return np.asfortranarray(_blas.dgemm(1.0, A, B, trans_a=1))


def _sub_prod(C: np.ndarray, A: np.ndarray, B: np.ndarray) -> None:
    """C -= A @ B in place (dgemm('N','N', alpha=-1, beta=1))."""
    if A.shape[1] == 0 or C.size == 0:
        return
    out = _blas.dgemm(-1.0, A, B, beta=1.0, c=C, overwrite_c=1)
    if out is not C and not np.shares_memory(out, C):
        C[...] = out


def _trsm_right_upper(B: np.ndarray, T: np.ndarray) -> None:
    """B := B T^{-1}, T upper, non-unit (dtrsm 'R','U','N','N')."""
    if B.size == 0:
        return
    out = _blas.dtrsm(1.0, T, B, side=1, lower=0, trans_a=0, diag=0, overwrite_b=1)
    if out is not B and not np.shares_memory(out, B):
        B[...] = out


def _trsm_left_upper_trans(T: np.ndarray, B: np.ndarray) -> None:
    """B := T^{-T} B, T upper, non-unit (dtrsm 'L','U','T','N')."""
    if B.size == 0:
        return
    out = _blas.dtrsm(1.0, T, B, side=0, lower=0, trans_a=1, diag=0, overwrite_b=1)
    if out is not B and not np.shares_memory(out, B):
        B[...] = out


def _chol_upper(M: np.ndarray) -> tuple[np.ndarray, int]:
    """dpotrf('U') of the upper triangle of M; strictly-lower part zeroed.

    Mirrors ``dlaset(LOWER)+dlacpy(UPPER)+dpotrf(UPPER)`` in the reference
    (e.g. SRC/orth.c:162-171). On breakdown LAPACK leaves a partial factor,
    which is returned together with info > 0.
    """
    A = np.triu(np.asfortranarray(M, dtype=np.float64))
    c, info = _lapack.dpotrf(A, lower=0, clean=1, overwrite_a=1)
    return np.asfortranarray(c), int(info)


def tsqr_explicit(A: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Explicit thin QR of a tall panel (restates TSQR factorExplicit).

    Used where the reference calls ``mytsqr.factorExplicit`` (SRC/orth.c:107,
    271, 413, 505, 522, 534, 601, 613, 651).
    """
    m, n = A.shape
    if n == 0:
        return np.zeros((m, 0), order="F"), np.zeros((0, 0), order="F")
    qr, tau, _work, _info = _lapack.dgeqrf(np.array(A, order="F", copy=True))
    R = np.triu(qr[:n, :n])
    q, _work, _info = _lapack.dorgqr(qr, tau)
    return np.asfortranarray(q[:, :n]), np.asfortranarray(R)


def cholqr2_explicit(A: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """CholeskyQR2 of a tall panel: twice G = V^T V (dgemm 'T','N'),
    T = chol(G) (dpotrf 'U'), V = V T^{-1} (dtrsm 'R','U','N','N'); R = T2 T1.

    Not in the reference, which factors every panel with TSQR; this restates the
    published algorithm (Fukaya, Nakatsukasa, Yanagisawa, Yamamoto, "CholeskyQR2",
    2014) for the library's CholQR2 IntraOrtho option. A Cholesky breakdown
    carries on with the partial factor, as the reference does with dpotrf.
    """
    V = np.array(A, order="F", copy=True)
    Ts = []
    for _ in range(2):
        T, _info = _chol_upper(_gram(V, V))
        _trsm_right_upper(V, T)
        Ts.append(T)
    return V, np.asfortranarray(np.triu(Ts[1] @ Ts[0]))


def tsqr_tree_explicit(A: np.ndarray, TR: int = 256) -> tuple[np.ndarray, np.ndarray]:
    """Explicit thin QR by a TSQR reduction tree: Householder QR (LAPACK) of each
    TR-row tile, then of the stack of the tiles' R factors the same way, until one
    tile remains; the root's diag(R) made >= 0; Q by the down-sweep. The shape of
    the library's GPU TSQR, restated to show how a panel's Q depends on the tree
    when the panel is numerically rank deficient (for full-rank panels every
    explicit QR agrees up to column signs)."""
    m, n = A.shape
    if m <= TR:
        Q, R = np.linalg.qr(A)
        d = np.sign(np.diag(R))
        d[d == 0] = 1
        return np.asfortranarray(Q * d), np.asfortranarray(R * d[:, None])
    Qs, Rs = [], []
    for r0 in range(0, m, TR):
        t = A[r0:r0 + TR]
        h = t.shape[0]
        if h < n:
            t = np.vstack([t, np.zeros((n - h, n))])
        q, r = np.linalg.qr(t)
        Qs.append(q[:h])
        Rs.append(r)
    Qr, R = tsqr_tree_explicit(np.vstack(Rs), TR)
    Q = np.vstack([Qs[i] @ Qr[i * n:(i + 1) * n] for i in range(len(Qs))])
    return np.asfortranarray(Q), np.asfortranarray(R)


_INTRA = {"tsqr": tsqr_explicit, "cholqr2": cholqr2_explicit, "tsqr_tree": tsqr_tree_explicit}
_intra_fn = [tsqr_explicit]


def _intra_qr(A: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """The IntraOrtho in force for this run (TSQR, as in the reference, unless
    run_variant was asked for CholQR2)."""
    return _intra_fn[0](A)


def _nblocks(n: int, s: int) -> int:
    """p = ceil((n - s0)/s) with s0 = s (SRC/orth.c:55)."""
    return int(math.ceil((n - s) / float(s)))


def _check(X: np.ndarray, n: int, s: int, R: np.ndarray) -> None:
    if X.dtype != np.float64 or not X.flags.f_contiguous:
        raise ValueError("X must be a Fortran-ordered float64 array")
    if X.shape[1] < n:
        raise ValueError("X has fewer than n columns")
    if R.shape[0] < n or R.shape[1] < n or not R.flags.f_contiguous:
        raise ValueError("R must be a Fortran-ordered n x n array")
    if s < 1 or n < 2 * s:
        raise ValueError("the reference requires n >= 2s (SRC/orth.c:52)")


def _first_block(X: np.ndarray, s: int, R: np.ndarray) -> None:
    """IntraOrtho of block 1: dlacpy to Usub, TSQR into X[:, :s] and R[:s,:s].

    SRC/orth.c:105-107 (same in every variant).
    """
    Q1, R11 = _intra_qr(X[:, :s])
    X[:, :s] = Q1
    R[:s, :s] = R11


# --------------------------------------------------------------------------
# C1  bcgsi2P1s  (SRC/orth.c:48-222): one-sync Pythagorean BCGSI+P-1S
# --------------------------------------------------------------------------
def bcgsi2P1s(X: np.ndarray, n: int, s: int, R: np.ndarray) -> int:
    _check(X, n, s, R)
    s0 = s
    p = _nblocks(n, s)
    info_first = 0
    _first_block(X, s0, R)                                   # :105-107

    # First step (:110-147).
    ntemp = s + s0
    W = _gram(X[:, :ntemp], X[:, s0:s0 + s])                 # :111-114  [Q1 X2]^T X2
    W[s0:, :] -= W[:s0, :].T @ W[:s0, :]                     # :115-116  Omega - S^T S
    R[:s0, s0:s0 + s] = W[:s0, :]                            # :117
    Sdiag, inf = _chol_upper(W[s0:, :])                      # :118-119
    info_first = info_first or (inf and 1)
    _sub_prod(X[:, s0:s0 + s], X[:, :s0], W[:s0, :])         # :121-122
    _trsm_right_upper(X[:, s0:s0 + s], Sdiag)                # :123-124  U2
    nZ = min(s, n - s - s0)                                  # :125
    s2 = s + nZ
    # :127-131  [Q1 U2]^T [U2 X3] and X3^T X3 (s columns of X3, see module doc)
    G = _gram(X[:, :ntemp], X[:, s0:s0 + s2])
    Omega3_s = _gram(X[:, ntemp:ntemp + s], X[:, ntemp:ntemp + s])
    Yd_in = G[s0:ntemp, :s] - G[:s0, :s].T @ G[:s0, :s]      # :134-135
    Ydiag, inf = _chol_upper(Yd_in)                          # :136-137
    info_first = info_first or (inf and 1)
    _sub_prod(X[:, s0:s0 + s], X[:, :s0], G[:s0, :s])        # :139-140
    _trsm_right_upper(X[:, s0:s0 + s], Ydiag)                # :141-142  Q2
    R[:s0, s0:s0 + s] += G[:s0, :s] @ Sdiag                  # :144-145
    R[s0:s0 + s, s0:s0 + s] = Ydiag @ Sdiag                  # :146-147

    # The reference stores X3^T X3 with leading dimension s (:129-131) and reads
    # it back with leading dimension nZ in the first loop step (:160-163). When
    # nZ < s (2s < n < 3s) that read reinterprets the s*s buffer; reproduce it.
    Omega_flat = np.asfortranarray(Omega3_s).ravel(order="F")
    Omega = Omega_flat[: nZ * nZ].reshape((nZ, nZ), order="F").copy(order="F")

    mZ = s0
    info = info_first
    for i in range(1, p):
        mScol = mZ + s
        # :155-159  reconstruct S = Q_{1:k-1}^T X_k from the last reduced Gram.
        Scol = np.array(G[:mScol, s:s + nZ], order="F")
        Scol[mZ:mScol, :] -= G[:mZ, :s].T @ G[:mZ, s:s + nZ]
        _trsm_left_upper_trans(Ydiag, Scol[mZ:mScol, :])
        # :160-171  Pythagorean shift and Cholesky.
        Om = Omega - Scol.T @ Scol
        Sdiag, inf = _chol_upper(Om)
        if inf and not info:
            info = i + 1
        # :173-176  U_k = (X_k - Q S) Sdiag^{-1}.
        Xk = X[:, mScol:mScol + nZ]
        _sub_prod(Xk, X[:, :mScol], Scol)
        _trsm_right_upper(Xk, Sdiag)
        if i < p - 1:                                        # :177-190
            nZn = min(s, n - (i + 1) * s - s0)
            s2 = s + nZn
            ntemp = mScol + s
            G = _gram(X[:, :ntemp], X[:, mScol:mScol + s2])
            Omega = _gram(X[:, ntemp:ntemp + nZn], X[:, ntemp:ntemp + nZn])
            nY = s
        else:                                                # :191-199
            ntemp = mScol + nZ
            G = _gram(X[:, :ntemp], X[:, mScol:mScol + nZ])
            nY = nZ
            nZn = nZ
        # :200-204  Ydiag = chol(U^T U - Y^T Y).
        Ydiag, inf = _chol_upper(G[mScol:mScol + nY, :nY] - G[:mScol, :nY].T @ G[:mScol, :nY])
        if inf and not info:
            info = i + 1
        # :206-209  Q_k = (U_k - Q Y) Ydiag^{-1}.
        _sub_prod(Xk[:, :nY], X[:, :mScol], G[:mScol, :nY])
        _trsm_right_upper(Xk[:, :nY], Ydiag)
        # :211-215  R updates.
        R[:mScol, mScol:mScol + nY] = Scol[:, :nY] + G[:mScol, :nY] @ Sdiag
        R[mScol:mScol + nY, mScol:mScol + nY] = Ydiag @ Sdiag
        mZ += s
        nZ = nZn
    return info


# --------------------------------------------------------------------------
# C2  bcgsi21s  (SRC/orth.c:224-367): one-sync BCGSI+A-1S
# --------------------------------------------------------------------------
def bcgsi21s(X: np.ndarray, n: int, s: int, R: np.ndarray) -> int:
    _check(X, n, s, R)
    s0 = s
    p = _nblocks(n, s)
    info = 0
    _first_block(X, s0, R)                                   # :269-271

    ntemp = s + s0
    Scol = _gram(X[:, :s0], X[:, s0:s0 + s])                 # :275-278
    _sub_prod(X[:, s0:s0 + s], X[:, :s0], Scol)              # :280-281
    nZ = min(s, n - s - s0)                                  # :282
    s2 = s + nZ
    G = _gram(X[:, :ntemp], X[:, s0:s0 + s2])                # :284-287
    Ydiag, inf = _chol_upper(G[s0:ntemp, :s] - G[:s0, :s].T @ G[:s0, :s])  # :288-291
    info = info or (inf and 1)
    _sub_prod(X[:, s0:s0 + s], X[:, :s0], G[:s0, :s])        # :293-294
    _trsm_right_upper(X[:, s0:s0 + s], Ydiag)                # :295-296
    R[:s0, s0:s0 + s] = Scol + G[:s0, :s]                    # :298-301 (daxpy)
    R[s0:s0 + s, s0:s0 + s] = np.triu(Ydiag)                 # :302

    mZ = s0
    for i in range(1, p):
        mScol = mZ + s
        Scol = np.array(G[:mScol, s:s + nZ], order="F")      # :310
        Scol[mZ:mScol, :] -= G[:mZ, :s].T @ G[:mZ, s:s + nZ] # :311-312
        _trsm_left_upper_trans(Ydiag, Scol[mZ:mScol, :])     # :313-314
        Xk = X[:, mScol:mScol + nZ]
        _sub_prod(Xk, X[:, :mScol], Scol)                    # :323-324  (no scaling)
        if i < p - 1:                                        # :325-335
            nZn = min(s, n - (i + 1) * s - s0)
            s2 = s + nZn
            ntemp = mScol + s
            G = _gram(X[:, :ntemp], X[:, mScol:mScol + s2])
            nY = s
        else:                                                # :336-344
            ntemp = mScol + nZ
            G = _gram(X[:, :ntemp], X[:, mScol:mScol + nZ])
            nY = nZ
            nZn = nZ
        Ydiag, inf = _chol_upper(G[mScol:mScol + nY, :nY] - G[:mScol, :nY].T @ G[:mScol, :nY])  # :345-349
        if inf and not info:
            info = i + 1
        _sub_prod(Xk[:, :nY], X[:, :mScol], G[:mScol, :nY])  # :351-352
        _trsm_right_upper(Xk[:, :nY], Ydiag)                 # :353-354
        R[:mScol, mScol:mScol + nY] = Scol[:, :nY] + G[:mScol, :nY]   # :356-359
        R[mScol:mScol + nY, mScol:mScol + nY] = np.triu(Ydiag)       # :360
        mZ += s
        nZ = nZn
    return info


# --------------------------------------------------------------------------
# C3  bcgspipi2  (SRC/orth.c:369-462): two-sync BCGS-PIPI+
# --------------------------------------------------------------------------
def bcgspipi2(X: np.ndarray, n: int, s: int, R: np.ndarray) -> int:
    _check(X, n, s, R)
    s0 = s
    p = _nblocks(n, s)
    info = 0
    _first_block(X, s0, R)                                   # :411-413
    mScol = s0
    for i in range(p):
        nZ = min(s, n - i * s - s0)                          # :419
        ntemp = mScol + nZ
        Sc = _gram(X[:, :ntemp], X[:, mScol:mScol + nZ])     # :421-424  [Q X_k]^T X_k
        Sdiag, inf = _chol_upper(Sc[mScol:, :] - Sc[:mScol, :].T @ Sc[:mScol, :])  # :425-429
        if inf and not info:
            info = i + 1
        Xk = X[:, mScol:mScol + nZ]
        _sub_prod(Xk, X[:, :mScol], Sc[:mScol, :])           # :431-432
        _trsm_right_upper(Xk, Sdiag)                         # :433-434
        Yc = _gram(X[:, :ntemp], Xk)                         # :435-438  [Q U]^T U
        Ydiag, inf = _chol_upper(Yc[mScol:, :] - Yc[:mScol, :].T @ Yc[:mScol, :])  # :440-444
        if inf and not info:
            info = i + 1
        _sub_prod(Xk, X[:, :mScol], Yc[:mScol, :])           # :446-447
        _trsm_right_upper(Xk, Ydiag)                         # :448-449
        R[:mScol, mScol:mScol + nZ] = Sc[:mScol, :] + Yc[:mScol, :] @ Sdiag  # :451-453
        R[mScol:mScol + nZ, mScol:mScol + nZ] = Ydiag @ Sdiag                # :454-455
        mScol += s
    return info


# --------------------------------------------------------------------------
# C4  bcgsi2  (SRC/orth.c:464-548): BCGSI+ (BCGS2) with TSQR intra-ortho
# --------------------------------------------------------------------------
def bcgsi2(X: np.ndarray, n: int, s: int, R: np.ndarray) -> int:
    _check(X, n, s, R)
    s0 = s
    p = _nblocks(n, s)
    _first_block(X, s0, R)                                   # :503-505
    mScol = s0
    for i in range(p):
        nZ = min(s, n - i * s - s0)                          # :511
        Xk = X[:, mScol:mScol + nZ]
        S = _gram(X[:, :mScol], Xk)                          # :512-515
        _sub_prod(Xk, X[:, :mScol], S)                       # :518-519
        Qk, Sdiag = _intra_qr(Xk)                        # :520-523
        Xk[...] = Qk
        Y = _gram(X[:, :mScol], Xk)                          # :524-527
        _sub_prod(Xk, X[:, :mScol], Y)                       # :530-531
        Qk, Ydiag = _intra_qr(Xk)                        # :532-535
        Xk[...] = Qk
        R[:mScol, mScol:mScol + nZ] = S + Y @ Sdiag          # :537-539
        R[mScol:mScol + nZ, mScol:mScol + nZ] = Ydiag @ Sdiag  # :540-541
        mScol += s
    return 0


# --------------------------------------------------------------------------
# C5  bcgsi2P2s  (SRC/orth.c:550-697): TSQR first pass + one Pythagorean sync
# --------------------------------------------------------------------------
def bcgsi2P2s(X: np.ndarray, n: int, s: int, R: np.ndarray) -> int:
    _check(X, n, s, R)
    s0 = s
    p = _nblocks(n, s)
    info = 0
    _first_block(X, s0, R)                                   # :599-601

    ntemp = s + s0
    S12 = _gram(X[:, :s0], X[:, s0:s0 + s])                  # :605-608
    R[:s0, s0:s0 + s] = S12                                  # :609
    _sub_prod(X[:, s0:s0 + s], X[:, :s0], S12)               # :610-611
    Qk, Sdiag = _intra_qr(X[:, s0:s0 + s])               # :612-614
    X[:, s0:s0 + s] = Qk
    nZ = min(s, n - s - s0)                                  # :615
    s2 = s + nZ
    G = _gram(X[:, :ntemp], X[:, s0:s0 + s2])                # :617-620
    Ydiag, inf = _chol_upper(G[s0:ntemp, :s] - G[:s0, :s].T @ G[:s0, :s])  # :621-624
    info = info or (inf and 1)
    _sub_prod(X[:, s0:s0 + s], X[:, :s0], G[:s0, :s])        # :625-626
    _trsm_right_upper(X[:, s0:s0 + s], Ydiag)                # :627-628
    R[:s0, s0:s0 + s] += G[:s0, :s] @ Sdiag                  # :630-631
    R[s0:s0 + s, s0:s0 + s] = Ydiag @ Sdiag                  # :632-633

    mZ = s0
    for i in range(1, p):
        mScol = mZ + s
        Scol = np.array(G[:mScol, s:s + nZ], order="F")      # :641
        Scol[mZ:mScol, :] -= G[:mZ, :s].T @ G[:mZ, s:s + nZ] # :642-643
        _trsm_left_upper_trans(Ydiag, Scol[mZ:mScol, :])     # :644-645
        Xk = X[:, mScol:mScol + nZ]
        _sub_prod(Xk, X[:, :mScol], Scol)                    # :647-648
        Qk, Sdiag = _intra_qr(Xk)                        # :649-652
        Xk[...] = Qk
        if i < p - 1:                                        # :653-666
            nZn = min(s, n - (i + 1) * s - s0)
            s2 = s + nZn
            ntemp = mScol + s
            G = _gram(X[:, :ntemp], X[:, mScol:mScol + s2])
            nY = s
        else:                                                # :667-675
            ntemp = mScol + nZ
            G = _gram(X[:, :ntemp], X[:, mScol:mScol + nZ])
            nY = nZ
            nZn = nZ
        Ydiag, inf = _chol_upper(G[mScol:mScol + nY, :nY] - G[:mScol, :nY].T @ G[:mScol, :nY])  # :676-680
        if inf and not info:
            info = i + 1
        _sub_prod(Xk[:, :nY], X[:, :mScol], G[:mScol, :nY])  # :681-682
        _trsm_right_upper(Xk[:, :nY], Ydiag)                 # :683-684
        R[:mScol, mScol:mScol + nY] = Scol[:, :nY] + G[:mScol, :nY] @ Sdiag  # :686-688
        R[mScol:mScol + nY, mScol:mScol + nY] = Ydiag @ Sdiag                # :689-690
        mZ += s
        nZ = nZn
    return info


VARIANTS = {
    "bcgsi2P1s": bcgsi2P1s,
    "bcgsi21s": bcgsi21s,
    "bcgspipi2": bcgspipi2,
    "bcgsi2": bcgsi2,
    "bcgsi2P2s": bcgsi2P2s,
}


def run_variant(name: str, X0: np.ndarray, n: int, s: int, intra: str = "tsqr"):
    """Run one variant on a copy of X0 (m x n). Returns (Q, R, info).

    intra: "tsqr" (the reference's IntraOrtho, restated as LAPACK Householder QR),
    "tsqr_tree" (a TSQR reduction tree) or "cholqr2"."""
    m = X0.shape[0]
    X = np.zeros((m, max(n + s, 3 * s)), order="F")
    X[:, :n] = X0[:, :n]
    R = np.zeros((n, n), order="F")
    _intra_fn[0] = _INTRA[intra]
    try:
        info = VARIANTS[name](X, n, s, R)
    finally:
        _intra_fn[0] = tsqr_explicit
    return np.array(X[:, :n], order="F"), R, info


# --------------------------------------------------------------------------
# Accuracy metrics (SRC/util.c:36-75 restated) plus the 2-norm forms.
# --------------------------------------------------------------------------
def loo_fro(Q: np.ndarray) -> float:
    """||Q^T Q - I||_F, the reference's loss-of-orthogonality (SRC/util.c:50-58)."""
    G = Q.T @ Q
    G[np.diag_indices_from(G)] -= 1.0
    return float(np.linalg.norm(G, "fro"))


def loo_2(Q: np.ndarray) -> float:
    """||I - Q^T Q||_2 (largest |eigenvalue| of the symmetric error)."""
    G = Q.T @ Q
    G[np.diag_indices_from(G)] -= 1.0
    G = 0.5 * (G + G.T)
    w = np.linalg.eigvalsh(G)
    return float(np.max(np.abs(w))) if w.size else 0.0


def residual_fro(X: np.ndarray, Q: np.ndarray, R: np.ndarray) -> float:
    """||Q R - X||_F, the reference's backward error (SRC/util.c:61-72)."""
    return float(np.linalg.norm(Q @ R - X, "fro"))


def rel_residual(X: np.ndarray, Q: np.ndarray, R: np.ndarray) -> float:
    """||X - Q R||_F / ||X||_F."""
    nx = float(np.linalg.norm(X, "fro"))
    return residual_fro(X, Q, R) / nx if nx > 0 else 0.0
