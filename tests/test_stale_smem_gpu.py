"""No kernel may read shared memory it did not write.

orth_gb300_poison_shared_memory fills every SM's shared memory with a NaN bit
pattern. A kernel that reads a shared-memory entry it never wrote (for instance a
product over a template width NC when the panel has nc < NC columns) then reads
NaN, and 0 * NaN turns the result into NaN. Each case here poisons shared memory,
runs a QR whose block size is below its kernels' template widths, and checks that
the result is finite and bit-identical to an unpoisoned run.
"""
import numpy as np
import pytest

from bcgs_gb300 import inputs, orth

pytestmark = pytest.mark.gpu


def _qr(torch, X, variant, s, prec, poison):
    m, n = X.shape
    st = torch.cuda.current_stream().cuda_stream
    dX = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
    dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    if poison:
        assert orth.poison_shared_memory(stream=st) == 0
    rc, status = orth.run_dev(variant, m, n, s, dX.data_ptr(), m, dR.data_ptr(), n, prec, st)
    assert rc == 0 and status["breakdown_step"] == 0
    return dX.cpu().numpy().T, dR.cpu().numpy().T


@pytest.mark.parametrize("prec", ["fp64", "split7"])
@pytest.mark.parametrize("variant,s", [("bcgsi2P1s", 4), ("bcgsi2", 4), ("bcgsi2P2s", 12), ("bcgspipi2", 4)])
def test_results_do_not_depend_on_shared_memory_leftovers(lib, prec, variant, s):
    torch = pytest.importorskip("torch")
    p = orth.FP64 if prec == "fp64" else orth.SPLIT_BF16
    m, n = 70000, 6 * s
    X = inputs.graded_host(m, n, 1e4, seed=s + 3)
    Q0, R0 = _qr(torch, X, variant, s, p, poison=False)
    Q1, R1 = _qr(torch, X, variant, s, p, poison=True)
    assert np.isfinite(Q1).all() and np.isfinite(R1).all()
    assert np.array_equal(Q0, Q1) and np.array_equal(R0, R1)
