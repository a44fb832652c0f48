"""GPU test of the row-sharded path (orth_gb300_run_sharded), FP64, all five
variants: two ranks, each its own process with its own rows of X, exchanging
through a host-staged gloo allgather, give Q (assembled from the ranks' rows)
and R bit-identical to a one-rank run; and the one-rank run agrees with the
single-GPU entry point within the FP64 parity tolerance.

The two ranks share this run's one GPU. No kernel waits on another rank: every
exchange happens on the host between kernel launches (the callback synchronizes
the stream, gathers through gloo, and copies back), so the ranks' kernels are
independent launches.
"""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

import bcgs_port as port
from bcgs_gb300 import inputs, orth
from helpers import U, VARIANTS, metric_ok, qr_tolerance, sign_normalize

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def _run_ranks(tmp_path, size, m, n, s, variants):
    port_ = _free_port()
    procs = []
    for r in range(size):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE=str(size), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port_), OMP_NUM_THREADS="2")
        out = str(tmp_path / f"w{size}_r{r}.npz")
        procs.append((out, subprocess.Popen([sys.executable, os.path.join(HERE, "sharded_worker.py"), out, str(m),
                                             str(n), str(s), ",".join(variants)],
                                            env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    outs = []
    for out, p in procs:
        log, _ = p.communicate(timeout=900)
        assert p.returncode == 0, log.decode(errors="replace")[-3000:]
        outs.append(np.load(out))
    return outs


def test_two_ranks_bit_identical_to_one(lib, tmp_path):
    m, n, s = 2 * 8192 + 1234, 64, 16      # 3 chunks (rank 0: 1, padded; rank 1: 2); ragged last tile
    one = _run_ranks(tmp_path, 1, m, n, s, VARIANTS)[0]
    two = _run_ranks(tmp_path, 2, m, n, s, VARIANTS)
    assert int(two[0]["row0"]) == 0 and int(two[1]["row0"]) == int(two[0]["msub"])
    assert int(two[0]["msub"]) + int(two[1]["msub"]) == m
    X = inputs.graded_host(m, n, 1e6, seed=17)
    p = (n - s) // s
    for v in VARIANTS:
        assert int(one[f"{v}/rc"]) == 0 and int(one[f"{v}/step"]) == 0
        for w in two:
            assert int(w[f"{v}/rc"]) == 0 and int(w[f"{v}/step"]) == 0
        Q2 = np.vstack([w[f"{v}/Q"] for w in two])
        assert np.array_equal(Q2, one[f"{v}/Q"]), v
        assert np.array_equal(two[0][f"{v}/R"], one[f"{v}/R"]), v
        assert np.array_equal(two[1][f"{v}/R"], one[f"{v}/R"]), v
        # The same number of synchronizations as the single-GPU path.
        expected = {"bcgspipi2": 2 * p, "bcgsi2": 2 * p}.get(v, p + 1)
        assert int(two[0][f"{v}/reductions"]) == expected == int(two[1][f"{v}/reductions"])
        # The sharded chunking against the single-GPU entry point and the oracle.
        Q, R = one[f"{v}/Q"], np.triu(one[f"{v}/R"])
        Qh, Rh, rc, _ = orth.qr(v, X, s)
        assert rc == 0
        Qs, Rs = sign_normalize(Q, R)
        Qhs, Rhs = sign_normalize(Qh, Rh)
        tol = qr_tolerance(1e6)
        assert np.max(np.abs(Qs - Qhs)) <= tol and np.max(np.abs(Rs - Rhs)) <= tol * np.max(np.abs(Rhs))
        Qp, Rp, _ = port.run_variant(v, X, n, s)
        assert metric_ok(port.loo_2(Q), port.loo_2(Qp), n * U)
        assert metric_ok(port.rel_residual(X, Q, R), port.rel_residual(X, Qp, Rp), n * U)
