"""GPU tests of the split-precision (BF16 digit planes on tcgen05) path.

The split modes replace the FP64 tall products with exact products of BF16 digit
planes: 7 per operand (56-bit fixed point per column, SPLIT_BF16) or 6 (48-bit,
SPLIT_BF16_FAST). Checked here through the C ABI:
  * the tall Gram primitive (7 planes) against the FP64 Gram on ragged shapes;
  * full QRs of every variant: the 56-bit form within 10x of the FP64 path's LOO
    and residual; the 48-bit form at LOO_2 <= 1e-12 and residual <= 1e-12; both
    agreeing with the FP64 path's R;
  * bit-exact results run to run;
  * s = 32 and 64 blocks.
"""
import numpy as np
import pytest

import bcgs_port as port
from bcgs_gb300 import inputs, orth
from helpers import VARIANTS, sign_normalize

pytestmark = pytest.mark.gpu


def _dev(torch, X):
    return torch.from_numpy(np.ascontiguousarray(X.T)).cuda()      # (n, m) == X column-major


@pytest.mark.parametrize("shape", [(5000, 48, 16, 32), (33333, 200, 150, 40), (70000, 130, 100, 30),
                                   (1000, 20, 0, 7), (256, 64, 32, 32)])
def test_split_gram_matches_fp64(lib, shape):
    torch = pytest.importorskip("torch")
    m, na, b0, nb = shape
    n = max(na, b0 + nb)
    X = inputs.graded_host(m, n, 1e4, seed=m + na)
    dX = _dev(torch, X)
    Cs = torch.zeros((nb, na), dtype=torch.float64, device="cuda")   # na x nb col-major
    Cf = torch.zeros_like(Cs)
    st = torch.cuda.current_stream().cuda_stream
    assert orth.gram_dev(m, na, b0, nb, dX.data_ptr(), m, Cf.data_ptr(), na, orth.FP64, st) == 0
    assert orth.gram_dev(m, na, b0, nb, dX.data_ptr(), m, Cs.data_ptr(), na, orth.SPLIT_BF16, st) == 0
    Cs, Cf = Cs.cpu().numpy().T, Cf.cpu().numpy().T
    norms = np.linalg.norm(X, axis=0)
    scale = np.outer(norms[:na], norms[b0:b0 + nb])
    rel = np.max(np.abs(Cs - Cf) / scale)
    # Digits scaled by the column max: the split Gram's error is below about
    # 2^-56 (max/rms)^2 of the norm product (max/rms is about 4-6 for these
    # columns); the bound also leaves room for the FP64 Gram's own rounding.
    assert rel < 2.0 ** -41, rel


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("kappa", [1e2, 1e6])
@pytest.mark.parametrize("mode", ["split7", "split6"])
def test_split_qr_accuracy(lib, variant, kappa, mode):
    torch = pytest.importorskip("torch")
    m, n, s = 100000, 96, 16
    X = inputs.graded_host(m, n, kappa, seed=11)
    st = torch.cuda.current_stream().cuda_stream
    out = {}
    split = orth.SPLIT_BF16 if mode == "split7" else orth.SPLIT_BF16_FAST
    for prec in (orth.FP64, split):
        dX = _dev(torch, X)
        dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        rc, status = orth.run_dev(variant, m, n, s, dX.data_ptr(), m, dR.data_ptr(), n, prec, st)
        assert rc == 0 and status["breakdown_step"] == 0 and status["timeout"] == 0, (rc, status)
        out[prec] = (dX.cpu().numpy().T.copy(), dR.cpu().numpy().T.copy())
    Q, R = out[split]
    Qf, Rf = out[orth.FP64]
    loo = port.loo_2(Q)
    res = port.rel_residual(X, Q, np.triu(R))
    loo_f = port.loo_2(Qf)
    res_f = port.rel_residual(X, Qf, np.triu(Rf))
    if mode == "split7":
        # 56-bit digits: the FP64 parity rule, within 10x of the FP64 path's LOO and
        # residual (floor 1e-15, about 10 u).
        assert loo <= 10 * max(loo_f, 1e-15), (loo, loo_f)
        assert res <= 10 * max(res_f, 1e-15), (res, res_f)
    else:
        # 48-bit digits: the accuracy target LOO <= 1e-12, except where the variant
        # itself loses orthogonality in FP64 (bcgsi21s at high kappa).
        assert loo <= max(1e-12, 200 * loo_f), (loo, loo_f)
        assert res <= 1e-12, res
    Qs, Rs = sign_normalize(Q, np.triu(R))
    Qfs, Rfs = sign_normalize(Qf, np.triu(Rf))
    assert np.max(np.abs(Rs - Rfs)) <= 1e-10 * kappa * np.max(np.abs(Rfs))


def test_split_bit_exact_run_to_run(lib):
    torch = pytest.importorskip("torch")
    m, n, s = 60000, 64, 16
    X = inputs.graded_host(m, n, 1e5, seed=4)
    st = torch.cuda.current_stream().cuda_stream
    res = []
    for _ in range(2):
        dX = _dev(torch, X)
        dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        rc, _ = orth.run_dev("bcgsi2P1s", m, n, s, dX.data_ptr(), m, dR.data_ptr(), n, orth.SPLIT_BF16, st)
        assert rc == 0
        res.append((dX.cpu().numpy(), dR.cpu().numpy()))
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("s", [32, 64])
def test_split_wide_blocks(lib, variant, s):
    """s = 32 and 64 (config-3 block sizes): the update writes its output columns in
    groups of 32 over one digit store; the 56-bit form stays within 10x of FP64."""
    torch = pytest.importorskip("torch")
    m, n = 60000, 4 * s
    X = inputs.graded_host(m, n, 1e6, seed=s + 1)
    st = torch.cuda.current_stream().cuda_stream
    assert orth.split_supported(m, n, s)
    out = {}
    for prec in (orth.FP64, orth.SPLIT_BF16):
        dX = _dev(torch, X)
        dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        rc, status = orth.run_dev(variant, m, n, s, dX.data_ptr(), m, dR.data_ptr(), n, prec, st)
        assert rc == 0 and status["breakdown_step"] == 0 and status["timeout"] == 0, (rc, status)
        out[prec] = (dX.cpu().numpy().T.copy(), dR.cpu().numpy().T.copy())
    (Q, R), (Qf, Rf) = out[orth.SPLIT_BF16], out[orth.FP64]
    assert port.loo_2(Q) <= 10 * max(port.loo_2(Qf), 1e-15)
    assert port.rel_residual(X, Q, np.triu(R)) <= 10 * max(port.rel_residual(X, Qf, np.triu(Rf)), 1e-15)


@pytest.mark.parametrize("variant", ["bcgsi2P1s", "bcgsi21s", "bcgsi2"])
@pytest.mark.parametrize("spike", [1e3, 1e6])
def test_split_spiky_rows(lib, variant, spike):
    """Columns dominated by a few rows (a graded X whose first 64 rows are scaled by
    `spike`). The digit planes are fixed point scaled by each column's maximum, so
    the other rows keep fewer significant bits: the 56-bit form's residual rises
    to about 3-5e-14 here (measured 2.6e-14 to 5.1e-14 at spike 1e3 and 1e6, the
    FP64 path below 1e-15), while its orthogonality stays within 10x of FP64's.
    Checked: the same breakdown step as FP64, LOO_2 within 10x of FP64's, and the
    residual within the split form's accuracy target (1e-12)."""
    torch = pytest.importorskip("torch")
    m, n, s = 200000, 96, 16
    X = inputs.graded_host(m, n, 1e4, seed=17)
    X[:64, :] *= spike
    st = torch.cuda.current_stream().cuda_stream
    out = {}
    for prec in (orth.FP64, orth.SPLIT_BF16):
        dX = _dev(torch, X)
        dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        rc, status = orth.run_dev(variant, m, n, s, dX.data_ptr(), m, dR.data_ptr(), n, prec, st)
        assert rc == 0 and status["timeout"] == 0, (rc, status)
        out[prec] = (status["breakdown_step"], dX.cpu().numpy().T.copy(), dR.cpu().numpy().T.copy())
    (bs, Q, R), (bf, Qf, Rf) = out[orth.SPLIT_BF16], out[orth.FP64]
    assert bs == bf, (bs, bf)
    if bf == 0:
        assert port.loo_2(Q) <= 10 * max(port.loo_2(Qf), 1e-15), (port.loo_2(Q), port.loo_2(Qf))
        assert port.rel_residual(X, Q, np.triu(R)) <= 1e-12
