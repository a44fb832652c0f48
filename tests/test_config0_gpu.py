"""The reference's CPU-runnable configuration on the GPU, against the reference.

X = U diag(sigma) W^T, m = 100000, n = 200, s = 10, sigma from 1 to 1e-8, rebuilt
from its seed. tests/golden/config0_ref.npz holds what the reference's own code
(SRC/orth.c built by oracle/build_ref.sh) computed for BCGSI+ and BCGSI+P-1S on it:
R and the metrics. The GPU results, in FP64 and in the 56-bit split form, must
match R within the FP64 QR parity tolerance (sign-normalized rows) and the
reference's LOO and residual within 10x.
"""
import os

import numpy as np
import pytest

import bcgs_port as port
from bcgs_gb300 import inputs, orth
from helpers import qr_tolerance

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "config0_ref.npz")


@pytest.mark.parametrize("prec", ["fp64", "split7"])
@pytest.mark.parametrize("variant", ["bcgsi2", "bcgsi2P1s"])
def test_config0_matches_reference(lib, variant, prec):
    torch = pytest.importorskip("torch")
    g = np.load(GOLD)
    m, n, s, kappa, seed = int(g["m"]), int(g["n"]), int(g["s"]), float(g["kappa"]), int(g["seed"])
    X = inputs.graded_host(m, n, kappa, seed=seed)
    dX = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
    dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    p = orth.FP64 if prec == "fp64" else orth.SPLIT_BF16
    rc, st = orth.run_dev(variant, m, n, s, dX.data_ptr(), m, dR.data_ptr(), n, p,
                          torch.cuda.current_stream().cuda_stream)
    assert rc == 0 and st["breakdown_step"] == 0
    Q, R = dX.cpu().numpy().T, np.triu(dR.cpu().numpy().T)
    Rref = g[f"{variant}/R"]
    sign = np.sign(np.diag(R)) * np.sign(np.diag(Rref))
    assert np.max(np.abs(sign[:, None] * R - Rref)) <= qr_tolerance(kappa) * np.max(np.abs(Rref))
    assert port.loo_2(Q) <= 10 * max(float(g[f"{variant}/loo_2"]), 1e-15)
    assert port.rel_residual(X, Q, R) <= 10 * max(float(g[f"{variant}/rel_residual"]), 1e-15)
