"""Golden results of the reference's own code at its CPU-runnable configuration.

The configuration: X = U diag(sigma) W^T with m = 100000, n = 200 (20 blocks of
s = 10), U and W the Q factors of seeded Gaussian matrices and sigma log-spaced
from 1 to 1e-8. X is regenerated from the seed by bcgs_gb300.inputs.graded_host, so
only the results are stored. The reference (oracle/_ref, built from its sources by
oracle/build_ref.sh) factors it with bcgsi2 (BCGSI+) and bcgsi2P1s (BCGSI+P-1S).
Stored per variant: R (n x n), ||Q^T Q - I||_2, ||Q^T Q - I||_F and
||X - QR||_F / ||X||_F.

    python tests/golden/make_config0.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "one-synchronization-bcgs_gb300"))

import bcgs_port as port  # noqa: E402
import ref  # noqa: E402
from bcgs_gb300 import inputs  # noqa: E402

M, N, S, KAPPA, SEED = 100000, 200, 10, 1e8, 100
VARIANTS = ("bcgsi2", "bcgsi2P1s")


def main():
    if not ref.available():
        raise SystemExit("oracle/_ref/liborth_ref.so is not built (oracle/build_ref.sh)")
    X = inputs.graded_host(M, N, KAPPA, seed=SEED)
    out = {"m": M, "n": N, "s": S, "kappa": KAPPA, "seed": SEED}
    for v in VARIANTS:
        Q, R, rc = ref.run(v, X, N, S)
        assert rc == 0, (v, rc)
        out[f"{v}/R"] = np.triu(R)
        out[f"{v}/loo_2"] = port.loo_2(Q)
        out[f"{v}/loo_fro"] = port.loo_fro(Q)
        out[f"{v}/rel_residual"] = port.rel_residual(X, Q, np.triu(R))
        print(v, out[f"{v}/loo_2"], out[f"{v}/rel_residual"])
    np.savez_compressed(os.path.join(HERE, "config0_ref.npz"), **out)


if __name__ == "__main__":
    main()
