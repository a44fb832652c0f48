"""GPU tests of the allocation-free BCGSI+P-1S entry point.

orth_gb300_bcgsi2P1s_dev_noalloc serves callers that cannot call cudaMalloc:
code that runs inside another framework's memory pool or allocator callback
(where a stray cudaMalloc would bypass the pool's accounting or synchronize
the device at the wrong moment) and programs whose device memory is fixed at
start-up. All its scratch lives in one fixed array inside the library.

Checked through the C ABI:
  * two calls in a row give Q and R bit-identical to the allocating entry
    point (orth_gb300_run_dev): both run the same FP64 kernels with the same
    Gram chunking, so no tolerance is needed;
  * in a fresh process that never calls the allocating path, free device
    memory does not change across calls after the first;
  * a shape whose scratch exceeds the fixed array is rejected before any
    kernel runs: real buffers keep their sentinel values.
The file is named to be collected last.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from bcgs_gb300 import inputs, orth

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _dev_copy(torch, X):
    return torch.from_numpy(np.ascontiguousarray(X.T)).cuda()   # (n, m) == X column-major


def test_noalloc_bit_identical_to_allocating_entry_point(lib):
    torch = pytest.importorskip("torch")
    m, n, s, kappa = 200000, 128, 16, 1e6
    X = inputs.graded_host(m, n, kappa, seed=77)
    stream = torch.cuda.current_stream().cuda_stream

    dX = _dev_copy(torch, X)
    dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    rc, st = orth.run_dev("bcgsi2P1s", m, n, s, dX.data_ptr(), m, dR.data_ptr(), n, orth.FP64, stream)
    assert rc == 0 and st["breakdown_step"] == 0
    Q_ref = dX.cpu().numpy().T.copy()
    R_ref = dR.cpu().numpy().T.copy()

    for _ in range(2):
        dX2 = _dev_copy(torch, X)
        dR2 = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        rc, st = orth.bcgsi2P1s_dev_noalloc(m, n, s, dX2.data_ptr(), m, dR2.data_ptr(), n, stream)
        assert rc == 0, rc
        assert st["breakdown_step"] == 0 and st["cuda_error"] == 0
        assert np.array_equal(dX2.cpu().numpy().T, Q_ref)
        assert np.array_equal(np.triu(dR2.cpu().numpy().T), np.triu(R_ref))


_FRESH = textwrap.dedent("""
    import sys
    sys.path.insert(0, {pkg!r})
    import numpy as np
    import torch
    from bcgs_gb300 import inputs, orth
    m, n, s = 100000, 64, 16
    X = inputs.graded_host(m, n, 1e4, seed=5)
    x0 = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
    dX = torch.empty_like(x0)
    dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    frees, outs = [], []
    for k in range(3):
        dX.copy_(x0)
        dR.zero_()
        torch.cuda.synchronize()
        rc, status = orth.bcgsi2P1s_dev_noalloc(m, n, s, dX.data_ptr(), m, dR.data_ptr(), n, st)
        assert rc == 0 and status["breakdown_step"] == 0, (rc, status)
        torch.cuda.synchronize()
        frees.append(torch.cuda.mem_get_info()[0])
        outs.append((dX.cpu().numpy().copy(), dR.cpu().numpy().copy()))
    # The first call may load the library's device module (which holds the fixed
    # array); the calls after it allocate nothing.
    assert frees[1] == frees[2], frees
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[1][0], outs[2][0])
    assert np.array_equal(outs[0][1], outs[2][1])
    print("NOALLOC_FRESH_OK", frees)
""")


def test_noalloc_allocates_nothing_in_a_fresh_process(lib):
    pytest.importorskip("torch")
    code = _FRESH.format(pkg=os.path.join(ROOT, "one-synchronization-bcgs_gb300"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "NOALLOC_FRESH_OK" in r.stdout


def test_noalloc_rejects_oversized_shape(lib, capfd):
    torch = pytest.importorskip("torch")
    # Its TSQR tree alone (about 1.07 m doubles at s = 16) exceeds the fixed array.
    m, n, s = 1 << 21, 32, 16
    dX = torch.full((n, m), 7.0, dtype=torch.float64, device="cuda")
    dR = torch.full((n, n), -3.0, dtype=torch.float64, device="cuda")
    rc, _ = orth.bcgsi2P1s_dev_noalloc(m, n, s, dX.data_ptr(), m, dR.data_ptr(), n,
                                       torch.cuda.current_stream().cuda_stream)
    assert rc == orth.NOALLOC_TOO_LARGE
    assert "static workspace" in capfd.readouterr().err
    torch.cuda.synchronize()
    assert bool((dX == 7.0).all()) and bool((dR == -3.0).all())
