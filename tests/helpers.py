"""Shared test helpers: golden fixtures and sign-normalized comparisons."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bcgs_golden.npz")
U = np.finfo(np.float64).eps / 2
VARIANTS = ("bcgsi2P1s", "bcgsi21s", "bcgspipi2", "bcgsi2", "bcgsi2P2s")


def load_golden():
    z = np.load(GOLDEN, allow_pickle=False)
    cases = [str(c) for c in z["cases"]]
    out = {}
    for c in cases:
        xkey = str(z[f"{c}/xkey"])
        n = int(z[f"{c}/n"])
        d = {"X": np.asfortranarray(z[xkey][:, :n]), "n": n, "s": int(z[f"{c}/s"]),
             "cond": float(z[f"{c}/cond"]), "qstride": int(z["qstride"])}
        for v in VARIANTS:
            d[v] = {"R": z[f"{c}/{v}/R"], "Qrows": z[f"{c}/{v}/Qrows"], "rc": int(z[f"{c}/{v}/rc"]),
                    "info": int(z[f"{c}/{v}/info"]), "metrics": z[f"{c}/{v}/metrics"]}
        out[c] = d
    return out


def sign_normalize(Q: np.ndarray, R: np.ndarray):
    """Make diag(R) >= 0 by flipping matching rows of R and columns of Q.

    QR factors agree only up to column signs: the reference's TSQR does not
    force a sign (SRC/orth.c:107 passes no forceNonnegativeDiagonal)."""
    d = np.sign(np.diag(R)).copy()
    d[d == 0] = 1.0
    return Q * d, R * d[:, None]


def qr_tolerance(cond: float) -> float:
    """Max-entry tolerance for Q and R/||R|| differences between two backward
    stable FP64 QR factorizations of the same matrix."""
    return 200.0 * U * max(cond, 1.0) + 1e-13


def metric_ok(ours: float, ref: float, floor: float) -> bool:
    """The parity rule: within 10x of the reference's value, with an
    absolute floor at the unit-roundoff level."""
    return np.isfinite(ours) and ours <= 10.0 * max(ref, floor)
