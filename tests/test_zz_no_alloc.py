"""GPU test of the allocation-free BCGSI+P-1S entry point.

orth_gb300_bcgsi2P1s_dev_noalloc serves callers that cannot call cudaMalloc
(code inside another framework's memory pool or allocator callback, programs
whose device memory is fixed at start-up): all its scratch lives in one fixed
array inside the library. This test calls it through the C ABI twice in a row,
on fresh copies of the input, and checks Q and R against the allocating entry
point (orth_gb300_run_dev) within the tolerance the parity tests use. The file
is named to be collected last.
"""
import numpy as np
import pytest

from bcgs_gb300 import inputs, orth
from helpers import qr_tolerance, sign_normalize

pytestmark = pytest.mark.gpu


def _dev_copy(torch, X):
    return torch.from_numpy(np.ascontiguousarray(X.T)).cuda()   # (n, m) == X column-major


def test_noalloc_matches_allocating_entry_point(lib):
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
    tol = qr_tolerance(kappa)
    Qr, Rr = sign_normalize(Q_ref, R_ref)

    for _ in range(2):
        dX2 = _dev_copy(torch, X)
        dR2 = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        rc, st = orth.bcgsi2P1s_dev_noalloc(m, n, s, dX2.data_ptr(), m, dR2.data_ptr(), n, stream)
        assert rc == 0, rc
        assert st["breakdown_step"] == 0 and st["cuda_error"] == 0
        Q = dX2.cpu().numpy().T
        R = dR2.cpu().numpy().T
        Qs, Rs = sign_normalize(Q, R)
        assert np.max(np.abs(Qs - Qr)) <= tol
        assert np.max(np.abs(Rs - Rr)) <= tol * np.max(np.abs(Rr))


def test_noalloc_rejects_oversized_shape(lib, capfd):
    torch = pytest.importorskip("torch")
    m, n, s = 1 << 21, 512, 16          # its TSQR tree alone exceeds the fixed workspace
    rc, _ = orth.bcgsi2P1s_dev_noalloc(m, n, s, 0x1000, m, 0x1000, n,
                                       torch.cuda.current_stream().cuda_stream)
    assert rc == orth.NOALLOC_TOO_LARGE
    assert "static workspace" in capfd.readouterr().err
