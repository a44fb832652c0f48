"""GPU tests of the accuracy-metrics kernels (orth_gb300_accuracy_dev).

They are the device form of the reference's test_orth_accuracy (SRC/util.c:36-75):
||Q^T Q - I||_F, ||Q R - X||_F and ||X||_F. They are checked against sums formed in
numpy's extended precision (np.longdouble), on inputs where the metrics are far above
FP64 rounding, so that the check measures the kernels' arithmetic and not rounding
noise; for both Gram forms (FP64 and exact tensor-core digits); bit-exact run to run;
and on finished QRs against the oracle's own metric functions.
"""
import numpy as np
import pytest

import bcgs_port as port
from bcgs_gb300 import inputs, orth

pytestmark = pytest.mark.gpu


def _dev(torch, A):
    return torch.from_numpy(np.ascontiguousarray(A.T)).cuda()      # column-major on the device


def _perturbed_qr(m, n, seed, eps_q, eps_x):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((m, n)))
    Q = Q + eps_q * rng.standard_normal((m, n)) / np.sqrt(m)
    R = np.triu(rng.standard_normal((n, n)))
    X = Q @ R + eps_x * rng.standard_normal((m, n))
    return X, Q, R


def _longdouble_metrics(X, Q, R):
    Ql, Rl, Xl = Q.astype(np.longdouble), np.triu(R).astype(np.longdouble), X.astype(np.longdouble)
    E = Ql.T @ Ql - np.eye(Q.shape[1], dtype=np.longdouble)
    W = Ql @ Rl - Xl
    return (float(np.sqrt((E * E).sum())), float(np.sqrt((W * W).sum())), float(np.sqrt((Xl * Xl).sum())), E)


@pytest.mark.parametrize("gram", ["fp64", "split"])
@pytest.mark.parametrize("shape", [(3000, 40), (8000, 64), (777, 33)])
def test_metrics_match_extended_precision(lib, gram, shape):
    torch = pytest.importorskip("torch")
    m, n = shape
    X, Q, R = _perturbed_qr(m, n, seed=m + n, eps_q=1e-7, eps_x=1e-6)
    loo_ref, res_ref, x_ref, E_ref = _longdouble_metrics(X, Q, R)
    dX, dQ, dR = _dev(torch, X), _dev(torch, Q), _dev(torch, R)
    dE = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    prec = orth.FP64 if gram == "fp64" else orth.SPLIT_BF16
    st = torch.cuda.current_stream().cuda_stream
    rc, loo, res, xf = orth.accuracy_dev(m, n, dX.data_ptr(), m, dQ.data_ptr(), m, dR.data_ptr(), n, prec,
                                         dE.data_ptr(), n, st)
    assert rc == 0
    # Metrics of size 1e-7 .. 1e-6 against FP64 evaluation error of about 1e-14.
    assert abs(loo - loo_ref) <= 1e-6 * loo_ref, (loo, loo_ref)
    assert abs(res - res_ref) <= 1e-6 * res_ref, (res, res_ref)
    assert abs(xf - x_ref) <= 1e-14 * x_ref, (xf, x_ref)
    E = dE.cpu().numpy().T
    assert np.array_equal(E, E.T)
    assert np.max(np.abs(E - E_ref.astype(np.float64))) <= 1e-12


def test_metrics_gram_forms_agree_and_are_deterministic(lib):
    torch = pytest.importorskip("torch")
    m, n = 50000, 64
    X, Q, R = _perturbed_qr(m, n, seed=5, eps_q=1e-9, eps_x=1e-9)
    dX, dQ, dR = _dev(torch, X), _dev(torch, Q), _dev(torch, R)
    st = torch.cuda.current_stream().cuda_stream
    runs = {}
    for prec in (orth.FP64, orth.SPLIT_BF16):
        a = orth.accuracy_dev(m, n, dX.data_ptr(), m, dQ.data_ptr(), m, dR.data_ptr(), n, prec, stream=st)
        b = orth.accuracy_dev(m, n, dX.data_ptr(), m, dQ.data_ptr(), m, dR.data_ptr(), n, prec, stream=st)
        assert a[0] == 0 and a == b     # bit-identical run to run
        runs[prec] = a
    (_, lf, rf, xf), (_, ls, rs, xs) = runs[orth.FP64], runs[orth.SPLIT_BF16]
    assert abs(lf - ls) <= 1e-4 * lf
    assert rf == rs and xf == xs        # the residual does not depend on the Gram form


@pytest.mark.parametrize("variant", ["bcgsi2P1s", "bcgsi2"])
def test_metrics_of_a_finished_qr(lib, variant):
    torch = pytest.importorskip("torch")
    m, n, s = 40000, 64, 8
    X = inputs.graded_host(m, n, 1e6, seed=3)
    dX0 = _dev(torch, X)
    dQ = dX0.clone()
    dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    rc, _ = orth.run_dev(variant, m, n, s, dQ.data_ptr(), m, dR.data_ptr(), n, orth.FP64, st)
    assert rc == 0
    rc, loo, res, xf = orth.accuracy_dev(m, n, dX0.data_ptr(), m, dQ.data_ptr(), m, dR.data_ptr(), n,
                                         orth.SPLIT_BF16, stream=st)
    assert rc == 0
    Q, R = dQ.cpu().numpy().T, dR.cpu().numpy().T
    # The oracle's FP64 metric functions carry rounding noise of about
    # sqrt(n) u ||.||; the device metrics are at least that accurate.
    assert abs(loo - port.loo_fro(Q)) <= 2e-14 * np.sqrt(n)
    assert abs(res / xf - port.rel_residual(X, Q, R)) <= 2e-15
    assert loo < 1e-12 and res / xf < 1e-14


def test_metrics_reject_bad_arguments(lib):
    torch = pytest.importorskip("torch")
    d = torch.zeros((4, 100), dtype=torch.float64, device="cuda")
    p = d.data_ptr()
    assert orth.accuracy_dev(100, 4, p, 99, p, 100, p, 4)[0] == 2      # ldX < m
    assert orth.accuracy_dev(100, 4, p, 100, p, 100, p, 3)[0] == 2     # ldR < n
    assert orth.accuracy_dev(100, 4, p, 100, p, 100, p, 4, gram_precision=7)[0] == 4
