"""Generate the condition-number sweep fixture from the reference's own code.

Run where the reference sources exist and ``oracle/build_ref.sh`` has built
``oracle/_ref/liborth_ref.so``:

    python tests/golden/make_kappa_sweep.py

Cases (inputs are regenerated from their seeds by the tests, so X itself is not
stored):
  * the config-1 construction reduced to m = 2^17, n = 256, s = 16:
    X = U diag(sigma) W^T with sigma log-spaced from 1 to 1/kappa, for
    kappa in {1e2, 1e6, 1e10, 1e14};
  * the config-2 s-step monomial basis reduced to m = 2^17, n = 256, s = 8.

For every case and each of the five variants the reference runs on one rank
with zeroed work/R and zero column padding (oracle/ref.py's harness rules).
Stored per (case, variant): the reference's return code, the first Cholesky
breakdown step (1-based block step; 0 for none) as the restated oracle sees it
(the reference itself ignores dpotrf's info), the metrics
||Q^T Q - I||_F, ||Q^T Q - I||_2 and ||X - QR||_F / ||X||_F of the reference's
own Q and R, and |diag(R)|.
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

M = 1 << 17
N = 256
KAPPAS = (1e2, 1e6, 1e10, 1e14)


def cases():
    """(name, kind, kappa, m, n, s, seed)."""
    for i, k in enumerate(KAPPAS):
        yield f"graded_k{k:.0e}".replace("+", ""), "graded", k, M, N, 16, 1234 + i
    yield "monomial_s8", "monomial", 0.0, M, N, 8, 4321


def make_input(kind: str, kappa: float, m: int, n: int, s: int, seed: int) -> np.ndarray:
    if kind == "graded":
        return inputs.graded_host(m, n, kappa, seed=seed)
    return inputs.monomial_host(m, n, s, seed=seed)


def main():
    if not ref.available():
        raise SystemExit("oracle/_ref/liborth_ref.so is not built (oracle/build_ref.sh)")
    out, names = {}, []
    for name, kind, kappa, m, n, s, seed in cases():
        X = make_input(kind, kappa, m, n, s, seed)
        names.append(name)
        for key, val in (("kind", kind), ("kappa", kappa), ("m", m), ("n", n), ("s", s), ("seed", seed)):
            out[f"{name}/{key}"] = np.array(val)
        for v in ref.VARIANTS:
            Q, R, rc = ref.run(v, X, n, s)
            _, _, info = port.run_variant(v, X, n, s)
            with np.errstate(all="ignore"):
                finite = bool(np.all(np.isfinite(Q)))
                metrics = np.array([port.loo_fro(Q) if finite else np.inf,
                                    port.loo_2(Q) if finite else np.inf,
                                    port.rel_residual(X, Q, R) if finite else np.inf])
            out[f"{name}/{v}/rc"] = np.array(rc)
            out[f"{name}/{v}/info"] = np.array(info)
            out[f"{name}/{v}/metrics"] = metrics
            out[f"{name}/{v}/rdiag"] = np.abs(np.diag(R)).copy()
            print(f"{name:16s} {v:10s} rc={rc} breakdown={info:3d} loo_F={metrics[0]:.3e} "
                  f"loo_2={metrics[1]:.3e} res={metrics[2]:.3e}", flush=True)
    out["cases"] = np.array(names)
    path = os.path.join(HERE, "kappa_sweep.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
