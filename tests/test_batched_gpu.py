"""GPU tests of the batched BCGSI+P-1S plan (orth_gb300_batch_*).

Every matrix of a batch runs the single-matrix driver's operations with the same
operands and summation orders, so with the same Gram chunking its Q and R are
bit-identical to orth_gb300_run_dev's, which the parity tests pin to the
reference. Checked here on ragged batches (uneven m, s and p, kappa spread):
bit-exactness against the single path, with and without tuning; graph replays
bit-identical; per-matrix breakdown reports equal to the single path's; accuracy
against the oracle; argument checks.
"""
import numpy as np
import pytest

import bcgs_port as port
from bcgs_gb300 import inputs, orth

pytestmark = pytest.mark.gpu


def _batch(seed, count, m_lo=2000, m_hi=30000, p_hi=8, kappa_hi=1e8):
    rng = np.random.default_rng(seed)
    ms = np.exp(rng.uniform(np.log(m_lo), np.log(m_hi), count)).astype(int)
    ss = rng.choice([4, 8, 16], count)
    ps = rng.integers(2, p_hi + 1, count)
    ks = np.exp(rng.uniform(np.log(1e2), np.log(kappa_hi), count))
    mats = [inputs.graded_host(int(m), int(s * p), float(k), seed=seed * 1000 + b)
            for b, (m, s, p, k) in enumerate(zip(ms, ss, ps, ks))]
    return [int(x) for x in ms], [int(s * p) for s, p in zip(ss, ps)], [int(x) for x in ss], mats


def _to_dev(torch, mats):
    return [torch.from_numpy(np.ascontiguousarray(X.T)).cuda() for X in mats]


def _single(torch, X, s, rows):
    m, n = X.shape
    orth.set_gram_chunk_rows(rows)
    try:
        dX = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
        dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        rc, st = orth.run_dev("bcgsi2P1s", m, n, s, dX.data_ptr(), m, dR.data_ptr(), n, orth.FP64,
                              torch.cuda.current_stream().cuda_stream)
        assert rc == 0
        return dX.cpu().numpy().T, dR.cpu().numpy().T, st["breakdown_step"]
    finally:
        orth.set_gram_chunk_rows(0)


def _run_batch(torch, ms, ns, ss, mats, tune):
    dX = _to_dev(torch, mats)
    dR = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in ns]
    st = torch.cuda.current_stream().cuda_stream
    plan = orth.Batch(ms, ns, ss, [x.data_ptr() for x in dX], [r.data_ptr() for r in dR], tune=tune, stream=st)
    assert plan.rc == 0
    assert plan.run(st) == 0
    torch.cuda.synchronize()
    return plan, dX, dR


@pytest.mark.parametrize("tune", [False, True])
def test_batch_bit_exact_vs_single(lib, tune):
    torch = pytest.importorskip("torch")
    ms, ns, ss, mats = _batch(seed=7, count=24)
    plan, dX, dR = _run_batch(torch, ms, ns, ss, mats, tune)
    tuned = plan.info()["tuned"]
    rc, steps, _, _ = plan.status()
    assert rc == 0
    for b, X in enumerate(mats):
        rows = tuned[4 if ss[b] <= 4 else (8 if ss[b] <= 8 else 16)][1]
        Q1, R1, step1 = _single(torch, X, ss[b], rows)
        Qb, Rb = dX[b].cpu().numpy().T, dR[b].cpu().numpy().T
        assert np.array_equal(Qb, Q1), b
        assert np.array_equal(Rb, R1), b
        assert steps[b] == step1
    plan.close()


def test_batch_graph_replay_is_bit_identical(lib):
    torch = pytest.importorskip("torch")
    ms, ns, ss, mats = _batch(seed=11, count=16)
    plan, dX, dR = _run_batch(torch, ms, ns, ss, mats, tune=False)
    first = [(x.clone(), r.clone()) for x, r in zip(dX, dR)]
    for b, X in enumerate(mats):          # restore the inputs and replay the graph
        dX[b].copy_(torch.from_numpy(np.ascontiguousarray(X.T)))
        dR[b].zero_()
    assert plan.run(torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    for b in range(len(mats)):
        assert torch.equal(first[b][0], dX[b]) and torch.equal(first[b][1], dR[b])
    info = plan.info()
    assert info["graph_nodes"] >= info["launches"] > 0
    plan.close()


def test_batch_accuracy_vs_oracle(lib):
    torch = pytest.importorskip("torch")
    ms, ns, ss, mats = _batch(seed=3, count=12, m_hi=12000, p_hi=6, kappa_hi=1e6)
    plan, dX, dR = _run_batch(torch, ms, ns, ss, mats, tune=True)
    for b, X in enumerate(mats):
        Q, R = dX[b].cpu().numpy().T, dR[b].cpu().numpy().T
        Qo, Ro, _ = port.run_variant("bcgsi2P1s", X, ns[b], ss[b])
        lo, lq = port.loo_2(Qo), port.loo_2(Q)
        ro, rq = port.rel_residual(X, Qo, Ro), port.rel_residual(X, Q, R)
        assert lq <= max(10 * lo, 1e-14), (b, lq, lo)
        assert rq <= max(10 * ro, 1e-15), (b, rq, ro)
    plan.close()


def test_batch_reports_breakdowns_per_matrix(lib):
    torch = pytest.importorskip("torch")
    ms, ns, ss, mats = _batch(seed=5, count=6, m_hi=8000, p_hi=6, kappa_hi=1e4)
    # Matrix 2: rank deficient beyond FP64 (kappa 1e20) -> the Pythagorean
    # Cholesky breaks down; the others are well conditioned.
    mats[2] = inputs.graded_host(ms[2], ns[2], 1e20, seed=99)
    plan, dX, dR = _run_batch(torch, ms, ns, ss, mats, tune=False)
    rc, steps, infos, nbroken = plan.status()
    assert rc == 0
    for b, X in enumerate(mats):
        _, _, step1 = _single(torch, X, ss[b], 8192)
        assert steps[b] == step1, b
    assert steps[2] > 0 and nbroken >= 1
    assert all(steps[b] == 0 for b in (0, 1, 3, 4, 5))
    plan.close()


def test_batch_rejects_bad_arguments(lib):
    torch = pytest.importorskip("torch")
    x = torch.zeros((32, 3000), dtype=torch.float64, device="cuda")
    r = torch.zeros((32, 32), dtype=torch.float64, device="cuda")
    assert orth.Batch([3000], [32], [32], [x.data_ptr()], [r.data_ptr()]).rc == 2        # s > 16
    assert orth.Batch([3000], [32], [8], [x.data_ptr()], [r.data_ptr()], ldx=[2999]).rc == 2
    assert orth.Batch([3000], [32], [8], [x.data_ptr()], [r.data_ptr()], precision=7).rc == 4
    assert orth.Batch([3000], [32], [8], [x.data_ptr()], [r.data_ptr()], variant="bcgsi2").rc == 4


@pytest.mark.parametrize("variant,form", [("bcgsi2P1s", "staged"), ("bcgsi2P1s", "streams"),
                                          ("bcgsi21s", "streams")])
def test_split_batch_matches_single_split_runs(lib, variant, form):
    """Split-precision batches: BCGSI+P-1S with s <= 16 runs as staged graphs (one
    launch per stage for all matrices), other variants (or on request) through the
    single-matrix tensor-core driver per matrix. Either way each matrix's Q and R are
    bit-identical to orth_gb300_run_dev's, within 10x of the FP64 path's LOO and
    residual; breakdowns are reported per matrix; two runs give the same bits."""
    torch = pytest.importorskip("torch")
    ms, ns, ss, mats = _batch(seed=21, count=10, m_hi=20000, p_hi=6, kappa_hi=1e6)
    dX = _to_dev(torch, mats)
    dR = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in ns]
    st = torch.cuda.current_stream().cuda_stream
    plan = orth.Batch(ms, ns, ss, [x.data_ptr() for x in dX], [r.data_ptr() for r in dR],
                      precision=orth.SPLIT_BF16, stream=st, variant=variant, streams=(form == "streams"))
    assert plan.rc == 0
    if form == "staged":
        # launches per run: a few hundred per wave, not about a hundred per matrix per step
        assert 0 < plan.info()["launches"] < 400, plan.info()
    for rep in range(2):
        for b, X in enumerate(mats):
            dX[b].copy_(torch.from_numpy(np.ascontiguousarray(X.T)))
            dR[b].zero_()
        assert plan.run(st) == 0
        rc, steps, _, _ = plan.status()
        assert rc == 0
    _check_split_batch(torch, variant, ms, ns, ss, mats, dX, dR, steps, st)
    plan.close()


def _check_split_batch(torch, variant, ms, ns, ss, mats, dX, dR, steps, st):
    for b, X in enumerate(mats):
        m, n, s = ms[b], ns[b], ss[b]
        outs = {}
        for prec in (orth.SPLIT_BF16, orth.FP64):
            x1 = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
            r1 = torch.zeros((n, n), dtype=torch.float64, device="cuda")
            rc1, st1 = orth.run_dev(variant, m, n, s, x1.data_ptr(), m, r1.data_ptr(), n, prec, st)
            assert rc1 == 0
            outs[prec] = (x1.cpu().numpy().T, r1.cpu().numpy().T, st1["breakdown_step"])
        Qs, Rs, step_s = outs[orth.SPLIT_BF16]
        assert np.array_equal(dX[b].cpu().numpy().T, Qs), b
        assert np.array_equal(np.triu(dR[b].cpu().numpy().T), np.triu(Rs)), b
        assert steps[b] == step_s
        Qf, Rf, _ = outs[orth.FP64]
        if step_s == 0:
            assert port.loo_2(Qs) <= 10 * max(port.loo_2(Qf), 1e-15)
            assert port.rel_residual(X, Qs, np.triu(Rs)) <= 10 * max(port.rel_residual(X, Qf, np.triu(Rf)), 1e-15)


def test_split_staged_batch_several_waves(lib, monkeypatch):
    """A wave budget smaller than the batch (ORTH_GB300_SPLIT_WAVE_BYTES) splits the
    staged plan into several waves, replayed in order; every matrix is still
    bit-identical to its single run, including a p = 1 matrix (n = 2s) and
    breakdowns at high kappa."""
    torch = pytest.importorskip("torch")
    ms, ns, ss, mats = _batch(seed=5, count=9, m_hi=12000, p_hi=5, kappa_hi=1e10)
    ms.append(4000); ns.append(32); ss.append(16)
    mats.append(inputs.graded_host(4000, 32, 1e3, seed=99))
    est = orth.split_batch_dry_run(ms, ns, ss, 1 << 60)
    monkeypatch.setenv("ORTH_GB300_SPLIT_WAVE_BYTES", str(max(1, est["bytes"] // 3)))
    assert orth.split_batch_dry_run(ms, ns, ss, max(1, est["bytes"] // 3))["waves"] >= 3
    dX = _to_dev(torch, mats)
    dR = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in ns]
    st = torch.cuda.current_stream().cuda_stream
    plan = orth.Batch(ms, ns, ss, [x.data_ptr() for x in dX], [r.data_ptr() for r in dR],
                      precision=orth.SPLIT_BF16, stream=st)
    assert plan.rc == 0
    assert plan.run(st) == 0
    rc, steps, _, nbroken = plan.status()
    assert rc == 0
    _check_split_batch(torch, "bcgsi2P1s", ms, ns, ss, mats, dX, dR, steps, st)
    plan.close()
