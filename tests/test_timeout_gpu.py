"""GPU test of the failure path: a bounded device wait that runs out.

The tensor-core kernels wait on mbarriers with a 2 s limit; when one runs out, the
kernel records a code, sets its abort flag and returns instead of hanging. Here one
thread waits on an mbarrier that nothing completes (orth_gb300_timeout_probe). The
host reads the recorded code, and the context stays usable: a split-precision QR
run afterwards is correct and reports no timeout.
"""
import time

import pytest

import bcgs_port as port
from bcgs_gb300 import inputs, orth

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_reports(lib):
    t0 = time.perf_counter()
    rc, code, abort = orth.timeout_probe(4242)
    dt = time.perf_counter() - t0
    assert rc == 0 and code == 4242 and abort == 1
    assert 1.5 < dt < 30.0          # the 2 s limit, not an immediate return
    X = inputs.graded_host(20000, 64, 1e4, seed=2)
    assert orth.set_host_precision(orth.SPLIT_BF16) == 0
    try:
        Q, R, rc, st = orth.qr("bcgsi2P1s", X, 16)
    finally:
        orth.set_host_precision(orth.FP64)
    assert rc == 0 and st["timeout"] == 0 and st["cuda_error"] == 0
    assert port.loo_fro(Q) < 1e-13
