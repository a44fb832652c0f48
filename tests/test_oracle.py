"""CPU tests of the oracle: the numpy restatement against the golden fixtures
produced by the reference's own code, and (where built) the reference itself."""
import numpy as np
import pytest

import bcgs_port as port
import ref
from helpers import VARIANTS, load_golden, qr_tolerance, sign_normalize

GOLD = load_golden()


@pytest.mark.parametrize("case", sorted(GOLD))
@pytest.mark.parametrize("variant", VARIANTS)
def test_port_matches_reference_golden(case, variant):
    g = GOLD[case]
    X, n, s = g["X"], g["n"], g["s"]
    gv = g[variant]
    Q, R, info = port.run_variant(variant, X, n, s)
    assert info == gv["info"]
    if gv["info"] != 0:
        # The reference continues with a partial Cholesky factor; the restated
        # oracle follows it step for step, so results still agree where finite.
        fin = np.isfinite(gv["R"])
        assert np.array_equal(fin, np.isfinite(R))
        return
    Qs, Rs = sign_normalize(Q, R)
    Qg_rows = gv["Qrows"]
    Rg = gv["R"]
    d = np.sign(np.diag(Rg)).copy()
    d[d == 0] = 1
    Qg_rows, Rg = Qg_rows * d, Rg * d[:, None]
    tol = qr_tolerance(g["cond"])
    assert np.max(np.abs(Rs - Rg)) <= tol * np.max(np.abs(Rg))
    assert np.max(np.abs(Qs[:: g["qstride"], :] - Qg_rows)) <= tol
    loo_f, _, res = gv["metrics"]
    assert abs(port.loo_fro(Q) - loo_f) <= 0.5 * loo_f + 1e-15
    assert abs(port.rel_residual(X, Q, R) - res) <= 0.5 * res + 1e-16


@pytest.mark.skipif(not ref.available(), reason="oracle/_ref not built here")
@pytest.mark.parametrize("shape", [(700, 41, 6), (257, 24, 4), (1500, 64, 16), (400, 9, 3)])
@pytest.mark.parametrize("variant", VARIANTS)
def test_port_matches_reference_live(shape, variant):
    m, n, s = shape
    X = np.asfortranarray(np.random.default_rng(m + n + s).random((m, n)))
    Qr, Rr, rc = ref.run(variant, X, n, s)
    Qp, Rp, info = port.run_variant(variant, X, n, s)
    assert rc == 0
    if info:
        return
    Qr, Rr = sign_normalize(Qr, Rr)
    Qp, Rp = sign_normalize(Qp, Rp)
    tol = qr_tolerance(np.linalg.cond(X))
    assert np.max(np.abs(Qr - Qp)) <= tol
    assert np.max(np.abs(Rr - Rp)) <= tol * np.max(np.abs(Rr))


@pytest.mark.skipif(not ref.available(), reason="oracle/_ref not built here")
def test_reference_lwork_rule():
    X = np.asfortranarray(np.random.default_rng(0).random((100, 20)))
    _, _, rc = ref.run("bcgsi2P1s", X, 20, 5, lwork=ref.lwork_min(100, 20, 5) - 1)
    assert rc == 1


def test_metrics_of_exact_qr():
    X = np.asfortranarray(np.random.default_rng(1).standard_normal((300, 30)))
    Q, R = np.linalg.qr(X)
    assert port.loo_fro(Q) < 1e-14
    assert port.loo_2(Q) < 1e-14
    assert port.rel_residual(X, Q, R) < 1e-15


def test_graded_generator_condition():
    from bcgs_gb300 import inputs
    X = inputs.graded_host(2000, 40, 1e6, seed=5)
    c = np.linalg.cond(X)
    assert 0.9e6 < c < 1.1e6


def test_monomial_generator_blocks():
    from bcgs_gb300 import inputs
    X = inputs.monomial_host(512, 24, 8, seed=1)
    assert np.allclose(np.linalg.norm(X, axis=0), 1.0)
    # Block 2 starts from the last column of block 1.
    assert np.allclose(X[:, 8], X[:, 7])


def test_port_matches_reference_at_config0():
    """The restated oracle against the reference's own results at its CPU-runnable
    configuration (tests/golden/config0_ref.npz, made by make_config0.py)."""
    import os
    from bcgs_gb300 import inputs
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "config0_ref.npz"))
    m, n, s, kappa, seed = int(g["m"]), int(g["n"]), int(g["s"]), float(g["kappa"]), int(g["seed"])
    X = inputs.graded_host(m, n, kappa, seed=seed)
    for v in ("bcgsi2", "bcgsi2P1s"):
        Q, R, info = port.run_variant(v, X, n, s)
        R = np.triu(R)
        Rref = g[f"{v}/R"]
        sign = np.sign(np.diag(R)) * np.sign(np.diag(Rref))
        assert np.max(np.abs(sign[:, None] * R - Rref)) <= qr_tolerance(kappa) * np.max(np.abs(Rref))
        assert port.loo_2(Q) <= 10 * max(float(g[f"{v}/loo_2"]), 1e-15)


@pytest.mark.parametrize("variant", ["bcgsi2P1s", "bcgsi21s"])
def test_port_matches_kappa_sweep_fixture(variant):
    """The restated oracle against the reference's own results at kappa = 1e10 on
    the reduced config-1 construction (tests/golden/kappa_sweep.npz): the same
    breakdown step (P1s breaks down there), and where there is none, the same
    metrics."""
    import os
    from bcgs_gb300 import inputs
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kappa_sweep.npz"))
    case = "graded_k1e10"
    m, n, s, seed = (int(z[f"{case}/{k}"]) for k in ("m", "n", "s", "seed"))
    X = inputs.graded_host(m, n, float(z[f"{case}/kappa"]), seed=seed)
    Q, R, info = port.run_variant(variant, X, n, s)
    assert info == int(z[f"{case}/{variant}/info"])
    if info:
        return
    _, loo2, res = z[f"{case}/{variant}/metrics"]
    assert abs(port.loo_2(Q) - loo2) <= 0.5 * loo2
    assert abs(port.rel_residual(X, Q, R) - res) <= 0.5 * res


def test_cholqr2_restatement_is_a_qr():
    """The oracle's CholQR2 (the library's alternative IntraOrtho) gives the same
    factorization as its TSQR on a moderately conditioned panel."""
    from bcgs_gb300 import inputs
    A = inputs.graded_host(5000, 16, 1e4, seed=3)
    Qc, Rc = port.cholqr2_explicit(A)
    Qt, Rt = port.tsqr_explicit(A)
    assert np.all(np.diag(Rc) > 0)
    Qc, Rc = sign_normalize(Qc, Rc)
    Qt, Rt = sign_normalize(Qt, Rt)
    assert np.max(np.abs(Qc - Qt)) <= qr_tolerance(1e4)
    assert np.max(np.abs(Rc - Rt)) <= qr_tolerance(1e4) * np.max(np.abs(Rt))
    assert port.loo_2(Qc) < 1e-14


@pytest.mark.parametrize("variant", VARIANTS)
def test_port_cholqr2_variants(variant):
    from bcgs_gb300 import inputs
    X = inputs.graded_host(3000, 48, 1e5, seed=4)
    Q, R, info = port.run_variant(variant, X, 48, 8, intra="cholqr2")
    assert info == 0
    assert port.loo_2(Q) < 1e-13 and port.rel_residual(X, Q, R) < 1e-14


def test_p2s_breakdown_on_rank_deficient_panels_depends_on_the_tsqr():
    """On the s-step monomial basis the panels bcgsi2P2s hands to TSQR are
    numerically rank deficient; an explicit QR of such a panel is unique only up
    to its rounding noise, so the step at which the following Pythagorean pass
    breaks down depends on the TSQR implementation: the same restated algorithm
    breaks down at very different steps with LAPACK Householder QR (the stand-in
    for the reference's Trilinos TSQR) and with a 256-row TSQR tree (the GPU
    TSQR's shape). The GPU parity test therefore does not pin this step."""
    from bcgs_gb300 import inputs
    X = inputs.monomial_host(16384, 128, 8, seed=4321)
    _, _, step_lapack = port.run_variant("bcgsi2P2s", X, 128, 8)
    _, _, step_tree = port.run_variant("bcgsi2P2s", X, 128, 8, intra="tsqr_tree")
    assert step_lapack > 0 and step_tree > 0
    assert abs(step_lapack - step_tree) > 1, (step_lapack, step_tree)
    # For a full-rank panel both explicit QRs agree up to column signs.
    A = inputs.graded_host(4096, 16, 1e3, seed=1)
    Q1, R1 = sign_normalize(*port.tsqr_explicit(A))
    Q2, R2 = sign_normalize(*port.tsqr_tree_explicit(A))
    assert np.max(np.abs(Q1 - Q2)) <= qr_tolerance(1e3)
