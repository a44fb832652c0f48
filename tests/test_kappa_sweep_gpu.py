"""Parity across condition numbers: all five variants, FP64 and the 56-bit split
form, against the reference's own results (tests/golden/kappa_sweep.npz, made
by tests/golden/make_kappa_sweep.py from oracle/_ref).

Inputs are the config-1 construction reduced to m = 2^17, n = 256, s = 16 at
kappa in {1e2, 1e6, 1e10, 1e14}, and the config-2 monomial basis reduced to
m = 2^17, n = 256, s = 8, regenerated here from the fixture's seeds.

The rules (the reference's semantics, SRC/orth.c:160-171 and :200-204: dpotrf's
info is ignored and the loop carries on with the partial factor):
  * where the reference has no Cholesky breakdown: none here either, and
    ||I - Q^T Q||_2 and ||X - QR||_F / ||X||_F within 10x of the reference's
    (floor 1e-15, about 10 u); for kappa <= 1e6 also |diag(R)| within
    200 u kappa of the reference's, relative to max |diag(R)|;
  * where the reference breaks down: a breakdown here too, at the same block
    step within +-1. The step is the comparable quantity: after a breakdown
    both carry on with a partial factor, and Q is no longer a result.
One case is exempt from the step rule: bcgsi2P2s on the monomial basis. Its
panels go through TSQR (SRC/orth.c:649-652) while numerically rank deficient,
where an explicit QR is unique only up to rounding noise; the step of the
following Pythagorean breakdown then depends on the TSQR implementation
(the restated algorithm breaks down at step 13 with LAPACK QR and at step 5
with a TSQR tree on the same input: tests/test_oracle.py::
test_p2s_breakdown_on_rank_deficient_panels_depends_on_the_tsqr), and the
reference's TSQR (Trilinos) is not pinned. There the run must complete and
report its status.
Every call goes through the C ABI (orth_gb300_run_dev).
"""
import os

import numpy as np
import pytest

import bcgs_port as port
from bcgs_gb300 import inputs, orth
from helpers import U, VARIANTS

pytestmark = pytest.mark.gpu
FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kappa_sweep.npz")
Z = np.load(FIX, allow_pickle=False)
CASES = [str(c) for c in Z["cases"]]
_X = {}


def case_input(name):
    if name not in _X:
        kind = str(Z[f"{name}/kind"])
        m, n, s, seed = (int(Z[f"{name}/{k}"]) for k in ("m", "n", "s", "seed"))
        if kind == "graded":
            _X[name] = inputs.graded_host(m, n, float(Z[f"{name}/kappa"]), seed=seed)
        else:
            _X[name] = inputs.monomial_host(m, n, s, seed=seed)
    return _X[name]


@pytest.mark.parametrize("precision", ["fp64", "split7"])
@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("case", CASES)
def test_kappa_sweep_vs_reference(lib, case, variant, precision):
    torch = pytest.importorskip("torch")
    X = case_input(case)
    m, n = X.shape
    s = int(Z[f"{case}/s"])
    prec = orth.FP64 if precision == "fp64" else orth.SPLIT_BF16
    dX = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()       # (n, m) == X column-major
    dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    rc, st = orth.run_dev(variant, m, n, s, dX.data_ptr(), m, dR.data_ptr(), n, prec,
                          torch.cuda.current_stream().cuda_stream)
    assert rc == 0 and st["timeout"] == 0 and st["cuda_error"] == 0, (rc, st)
    ref_step = int(Z[f"{case}/{variant}/info"])
    if str(Z[f"{case}/kind"]) == "monomial" and variant == "bcgsi2P2s":
        return
    if ref_step != 0:
        assert st["breakdown_step"] > 0, (ref_step, st)
        assert abs(st["breakdown_step"] - ref_step) <= 1, (ref_step, st)
        return
    assert st["breakdown_step"] == 0, st
    Q = dX.cpu().numpy().T
    R = np.triu(dR.cpu().numpy().T)
    _, loo2_ref, res_ref = (float(x) for x in Z[f"{case}/{variant}/metrics"])
    loo2 = port.loo_2(Q)
    res = port.rel_residual(X, Q, R)
    assert loo2 <= 10.0 * max(loo2_ref, 1e-15), (loo2, loo2_ref)
    assert res <= 10.0 * max(res_ref, 1e-15), (res, res_ref)
    kappa = float(Z[f"{case}/kappa"])
    if str(Z[f"{case}/kind"]) == "graded" and kappa <= 1e6:
        rd = Z[f"{case}/{variant}/rdiag"]
        assert np.max(np.abs(np.abs(np.diag(R)) - rd)) <= 200 * U * kappa * np.max(rd)
