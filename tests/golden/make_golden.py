"""Generate the golden fixtures from the reference's own code (oracle/_ref).

Run in a container where the reference sources exist and ``oracle/build_ref.sh``
has built ``oracle/_ref/liborth_ref.so``:

    python tests/golden/make_golden.py

For every case the reference's five variants are run on one rank with zeroed
``work``/``R`` and zero column padding (the harness rules in oracle/ref.py).
Stored per case: the input X (shared by cases that factor its leading
columns), and per variant the full R, every 8th row of Q,
the reference's return code, the Cholesky breakdown step seen by the restated
oracle (the reference itself ignores dpotrf's info), and the metrics
||Q^T Q - I||_F, ||Q^T Q - I||_2 and ||X - QR||_F / ||X||_F.

Inputs are seeded numpy matrices. ``tc`` follows the reference's own test driver
(TESTS/test_orth.c:284-292: m = 550, n = 35..39, s = 5, uniform [0,1) entries);
the others use the graded and monomial constructions of bcgs_gb300.inputs.
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

QSTRIDE = 16


def cases():
    """(case name, input name, input matrix, n, s); X[:, :n] is factored."""
    Xtc = inputs.uniform_host(550, 39, seed=2024)
    for n in range(35, 40):
        yield f"tc_n{n}", "in_tc", Xtc, n, 5
    Xg = inputs.graded_host(1200, 44, 1e6, seed=7)
    yield "graded_k1e6", "in_graded", Xg, 44, 8
    Xe = inputs.graded_host(300, 20, 1e3, seed=11)
    yield "edge_n2s", "in_edge", Xe, 16, 8
    yield "edge_n2s_plus4", "in_edge", Xe, 20, 8
    Xm = inputs.monomial_host(1024, 40, 8, seed=3)
    yield "monomial_s8", "in_monomial", Xm, 40, 8


def main():
    if not ref.available():
        raise SystemExit("oracle/_ref/liborth_ref.so is not built (oracle/build_ref.sh)")
    out = {}
    names = []
    for name, xkey, Xfull, n, s in cases():
        out[xkey] = np.asfortranarray(Xfull)
        X = np.asfortranarray(Xfull[:, :n])
        m = X.shape[0]
        names.append(name)
        out[f"{name}/xkey"] = np.array(xkey)
        out[f"{name}/n"] = np.array(n)
        out[f"{name}/s"] = np.array(s)
        out[f"{name}/cond"] = np.array(np.linalg.cond(X))
        for v in ref.VARIANTS:
            Q, R, rc = ref.run(v, X, n, s)
            _, _, info = port.run_variant(v, X, n, s)
            out[f"{name}/{v}/R"] = R
            out[f"{name}/{v}/Qrows"] = Q[::QSTRIDE, :]
            out[f"{name}/{v}/rc"] = np.array(rc)
            out[f"{name}/{v}/info"] = np.array(info)
            with np.errstate(all="ignore"):
                out[f"{name}/{v}/metrics"] = np.array(
                    [port.loo_fro(Q), port.loo_2(Q) if np.all(np.isfinite(Q)) else np.nan,
                     port.rel_residual(X, Q, R)])
            print(f"{name:16s} {v:10s} rc={rc} info={info} metrics={out[f'{name}/{v}/metrics']}")
    out["cases"] = np.array(names)
    out["qstride"] = np.array(QSTRIDE)
    path = os.path.join(HERE, "bcgs_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
