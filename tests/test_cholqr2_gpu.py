"""GPU tests of the CholQR2 IntraOrtho option (orth_gb300_set_intra_ortho).

The reference factors its panels with Trilinos TSQR; CholQR2 is this library's
cheaper alternative for them (two Gram passes, each one deterministic
reduction). Checked through the C ABI against the oracle run with the same
IntraOrtho (oracle/bcgs_port.py, cholqr2_explicit): Q and R/||R|| entries within
200 u cond(X) + 1e-13 after sign normalization, LOO and residual within 10x of
the oracle's; and against the reference's TSQR-based results: the same
accuracy within 10x.
"""
import numpy as np
import pytest

import bcgs_port as port
from bcgs_gb300 import inputs, orth
from helpers import U, VARIANTS, metric_ok, qr_tolerance, sign_normalize

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "split7"])
@pytest.mark.parametrize("variant", VARIANTS)
def test_cholqr2_matches_oracle(lib, variant, precision):
    m, n, s, kappa = 40000, 96, 16, 1e6
    X = inputs.graded_host(m, n, kappa, seed=31)
    assert orth.set_intra_ortho(orth.INTRA_CHOLQR2) == 0
    assert orth.set_host_precision(orth.FP64 if precision == "fp64" else orth.SPLIT_BF16) == 0
    try:
        Q, R, rc, st = orth.qr(variant, X, s)
    finally:
        orth.set_intra_ortho(orth.INTRA_TSQR)
        orth.set_host_precision(orth.FP64)
    assert rc == 0 and st["breakdown_step"] == 0 and st["cuda_error"] == 0, (rc, st)
    Qp, Rp, info = port.run_variant(variant, X, n, s, intra="cholqr2")
    assert info == 0
    Qs, Rs = sign_normalize(Q, R)
    Qps, Rps = sign_normalize(Qp, Rp)
    tol = qr_tolerance(kappa)
    assert np.max(np.abs(Rs - Rps)) <= tol * np.max(np.abs(Rps))
    assert np.max(np.abs(Qs - Qps)) <= tol
    assert metric_ok(port.loo_2(Q), port.loo_2(Qp), n * U)
    assert metric_ok(port.rel_residual(X, Q, R), port.rel_residual(X, Qp, Rp), n * U)
    Qt, Rt, _ = port.run_variant(variant, X, n, s)          # the reference's TSQR
    assert metric_ok(port.loo_2(Q), port.loo_2(Qt), n * U)
    assert metric_ok(port.rel_residual(X, Q, R), port.rel_residual(X, Qt, Rt), n * U)


def test_cholqr2_one_reduction_per_pass(lib):
    """CholQR2 adds two reductions per panel: block 1 of BCGSI+P-1S costs two
    more synchronizations than with TSQR."""
    torch = pytest.importorskip("torch")
    m, n, s = 20000, 64, 16
    X = inputs.graded_host(m, n, 1e3, seed=2)
    counts = {}
    for mode in (orth.INTRA_TSQR, orth.INTRA_CHOLQR2):
        assert orth.set_intra_ortho(mode) == 0
        try:
            dX = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
            dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
            rc, st = orth.run_dev("bcgsi2P1s", m, n, s, dX.data_ptr(), m, dR.data_ptr(), n, orth.FP64,
                                  torch.cuda.current_stream().cuda_stream)
        finally:
            orth.set_intra_ortho(orth.INTRA_TSQR)
        assert rc == 0 and st["breakdown_step"] == 0
        counts[mode] = orth.last_reduction_count()
    assert counts[orth.INTRA_CHOLQR2] == counts[orth.INTRA_TSQR] + 2
