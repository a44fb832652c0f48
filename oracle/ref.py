"""ctypes binding to the reference's own SRC/orth.c built by ``build_ref.sh``.

TEST INFRASTRUCTURE ONLY (the oracle). ``oracle/_ref/liborth_ref.so`` is the
reference's unmodified code on one rank; it exists where the reference sources
were present at build time and is compiled for the host it was built on.

Harness rules that follow from the reference's behaviour:
  * ``work`` and ``R`` are zeroed before every call: bcgsi2P1s and bcgsi2P2s copy
    only the upper triangle into Sdiag/Ydiag without clearing the lower one
    (SRC/orth.c:118,136,623) and then multiply full matrices (:144-147,:632).
  * X gets at least ``n + s`` (and ``3s``) columns of zero padding: bcgsi2P1s
    reads ``s`` columns of the third block even when fewer exist
    (SRC/orth.c:129-131).
  * ``lwork`` is the reference's minimum, 5ns + 9s^2 + msub*n (SRC/orth.c:82),
    computed in 64-bit here and checked to fit the reference's ``int``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "liborth_ref.so")
VARIANTS = ("bcgsi2P1s", "bcgsi21s", "bcgspipi2", "bcgsi2", "bcgsi2P2s")

_lib = None


def available() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    try:
        _load()
    except OSError:
        return False
    return True


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        for name in VARIANTS:
            f = getattr(lib, name)
            f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int,
                          dp, ctypes.c_int, dp, ctypes.c_int]
            f.restype = ctypes.c_int
        _lib = lib
    return _lib


def lwork_min(m: int, n: int, s: int) -> int:
    """The reference's minimum lwork on one rank (SRC/orth.c:82)."""
    return 5 * n * s + 9 * s * s + m * n


def run(name: str, X0: np.ndarray, n: int, s: int, lwork: int | None = None):
    """Run the reference variant ``name`` on a copy of X0[:, :n].

    Returns (Q, R, rc) with rc the reference's return code.
    """
    lib = _load()
    m = X0.shape[0]
    ncols = max(n + s, 3 * s)
    X = np.zeros((m, ncols), order="F")
    X[:, :n] = X0[:, :n]
    R = np.zeros((n, n), order="F")
    lw = lwork_min(m, n, s) if lwork is None else lwork
    if lw >= 2**31 or m * ncols >= 2**31:
        raise ValueError("size exceeds the reference's 32-bit index range")
    work = np.zeros(max(lw, 1), dtype=np.float64)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = getattr(lib, name)(m, n, s, X.ctypes.data_as(dp), m, R.ctypes.data_as(dp), n,
                            work.ctypes.data_as(dp), lw)
    return np.array(X[:, :n], order="F"), R, int(rc)
