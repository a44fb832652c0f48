"""Seeded synthetic test matrices for the BCGS QR workloads.

Two constructions, both column-major float64:

* ``graded``: X = U diag(sigma) W^T, where U is the Q factor of a seeded
  standard-Gaussian m x n matrix, W the Q factor of a seeded Gaussian n x n
  matrix and sigma is log-spaced from 1 down to 1/kappa, so kappa(X) = kappa.
* ``monomial``: an s-step Krylov-style monomial basis. A = diag(a) with a
  log-spaced in [1e-3, 1] over the m rows and b a seeded Gaussian vector. Block
  j is [v, Av, ..., A^{s-1} v] with every column normalized, where v is the last
  column of block j-1 (v = b for the first block). The blocks become
  increasingly ill-conditioned.

Host versions use numpy's PCG64 generator; device versions (``*_device``) use
torch's CUDA generator and are meant for sizes that do not fit the host path
(m = 2^22 .. 2^23). The two paths do not produce the same bytes; parity at those
sizes is checked through properties of the result (orthogonality, residual).
"""
from __future__ import annotations

import numpy as np


def graded_host(m: int, n: int, kappa: float, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((m, n))
    U, _ = np.linalg.qr(G)
    W, _ = np.linalg.qr(rng.standard_normal((n, n)))
    sigma = np.logspace(0.0, -np.log10(kappa), n) if n > 1 else np.ones(1)
    return np.asfortranarray((U * sigma) @ W.T)


def monomial_host(m: int, n: int, s: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    a = np.logspace(-3.0, 0.0, m)
    v = rng.standard_normal(m)
    X = np.empty((m, n), order="F")
    j = 0
    while j < n:
        w = v / np.linalg.norm(v)
        for i in range(min(s, n - j)):
            X[:, j + i] = w
            w = a * w
            w = w / np.linalg.norm(w)
        v = X[:, j + min(s, n - j) - 1].copy()
        j += s
    return X


def uniform_host(m: int, n: int, seed: int = 0) -> np.ndarray:
    """Uniform [0, 1) entries, the distribution of the reference's own test
    driver (TESTS/test_orth.c:42-44), from a seeded numpy generator."""
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.random((m, n)))


def _torch():
    import torch
    return torch


def graded_device(m: int, n: int, kappa: float, seed: int = 0, device: str = "cuda:0"):
    """Device version of ``graded_host``: returns a torch tensor of shape (n, m)
    whose row-major storage is X column-major (ld = m).

    U is the Q factor of the seeded Gaussian G, formed by two rounds of
    Cholesky QR (a Gaussian m x n matrix with m >> n is well conditioned, so two
    rounds give orthonormality to rounding). Only the tall products run on the
    GPU (matmul); the n x n factorizations run on the host with numpy, so this
    needs no GPU linear-algebra library.
    """
    torch = _torch()
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    Ut = torch.randn((n, m), generator=g, device=device, dtype=torch.float64)   # U^T, row-major
    for _ in range(2):
        Gram = (Ut @ Ut.t()).cpu().numpy()
        L = np.linalg.cholesky(0.5 * (Gram + Gram.T))
        Linv = torch.from_numpy(np.linalg.inv(L)).to(device)
        Ut = Linv @ Ut                       # (L^{-1} U^T) == (U L^{-T})^T
    rng = np.random.default_rng(seed + 1)
    W, _ = np.linalg.qr(rng.standard_normal((n, n)))
    sigma = np.logspace(0.0, -np.log10(kappa), n) if n > 1 else np.ones(1)
    M = torch.from_numpy(np.ascontiguousarray((W * sigma).T)).to(device)   # diag(sigma) W^T
    # X^T = M^T U^T, written in row blocks of X (column blocks of X^T).
    Xt = torch.empty((n, m), device=device, dtype=torch.float64)
    step = 1 << 20
    Mt = M.t().contiguous()
    for r0 in range(0, m, step):
        r1 = min(m, r0 + step)
        Xt[:, r0:r1] = Mt @ Ut[:, r0:r1]
    del Ut
    return Xt


def monomial_device(m: int, n: int, s: int, seed: int = 0, device: str = "cuda:0"):
    torch = _torch()
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    a = torch.logspace(-3.0, 0.0, m, device=device, dtype=torch.float64)
    v = torch.randn((m,), generator=g, device=device, dtype=torch.float64)
    Xt = torch.empty((n, m), device=device, dtype=torch.float64)
    j = 0
    while j < n:
        w = v / torch.sqrt((v * v).sum())
        for i in range(min(s, n - j)):
            Xt[j + i] = w
            w = a * w
            w = w / torch.sqrt((w * w).sum())
        v = Xt[j + min(s, n - j) - 1].clone()
        j += s
    return Xt
