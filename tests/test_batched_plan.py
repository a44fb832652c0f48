"""CPU tests of the batched plan's schedule (orth_gb300_batch_dry_run).

The batched form lays each matrix's BCGSI+P-1S steps (SRC/orth.c:48-222) on a
common stage sequence: the TSQR tree of block 1 (one stage per level, the root
sign fixes, one per down-sweep level), the first step's six stages, and four per
later block step. A Gram stage is two launches (partials, fixed-order reduction).
"""
import numpy as np
import pytest

from bcgs_gb300 import orth


def _tsqr_levels(m, tr=256, s=8):
    levels, rows = 0, m
    while rows > tr:
        rows = -(-rows // tr) * s
        levels += 1
    return levels


def _expected(ms, ns, ss):
    L = max(_tsqr_levels(m, s=s) for m, s in zip(ms, ss))
    p = max((n - s + s - 1) // s for n, s in zip(ns, ss))
    stages = (L + 1) + 1 + L + 6 + 4 * (p - 1)
    grams = 2 + (p - 1)
    return stages, stages + grams


@pytest.mark.parametrize("case", [
    ([3000], [32], [8]),
    ([3000, 200000, 5000], [32, 256, 8], [8, 16, 4]),
    ([2000] * 5, [8, 16, 24, 32, 40], [4, 4, 4, 4, 4]),
])
def test_dry_run_stage_counts(lib, case):
    ms, ns, ss = case
    d = orth.batch_dry_run(ms, ns, ss)
    assert d["rc"] == 0
    assert (d["stages"], d["launches"]) == _expected(ms, ns, ss)
    assert d["bytes"] > 0


def test_dry_run_config4_size(lib):
    rng = np.random.default_rng(2024)
    B = 4096
    m = np.exp(rng.uniform(np.log(2000), np.log(200000), B)).astype(int)
    s = rng.choice([4, 8, 16], B)
    p = rng.integers(2, 17, B)
    d = orth.batch_dry_run(m.tolist(), (s * p).tolist(), s.tolist())
    assert d["rc"] == 0
    # 16 blocks at most: 15 block steps after the first; stays one graph of < 100 launches.
    assert d["launches"] < 100
    # Plan workspace is a small fraction of the batch's own 120 GB.
    assert d["bytes"] < 4e9


@pytest.mark.parametrize("bad", [
    ([3000], [64], [32]),      # s > 16
    ([3000], [12], [8]),       # n < 2s
    ([10], [16], [8]),         # m < n
    ([3000], [32], [0]),       # s < 1
])
def test_dry_run_rejects(lib, bad):
    assert orth.batch_dry_run(*bad)["rc"] == 2


def _config4_shapes(seed=2024, B=4096):
    rng = np.random.default_rng(seed)
    m = np.exp(rng.uniform(np.log(2000), np.log(200000), B)).astype(int)
    s = rng.choice([4, 8, 16], B)
    p = rng.integers(2, 17, B)
    return m.tolist(), (s * p).tolist(), s.tolist()


def test_split_batch_plan_longest_first_to_least_loaded(lib):
    ms, ns, ss = _config4_shapes()
    d = orth.split_batch_plan(ms, ns, ss, free_bytes=270 << 30)
    S, slot_of, order = d["slots"], d["slot_of"], d["order"]
    assert S == 16
    w = [m * n * n for m, n in zip(ms, ns)]
    # The enqueue order is by job weight m n^2, longest first, ties by index.
    assert sorted(order) == list(range(len(ms)))
    assert all((w[a], -a) >= (w[b], -b) for a, b in zip(order, order[1:]))
    # Replaying the order: every job goes to a least-loaded slot (lowest index on ties).
    load = [0] * S
    for b in order:
        k = min(range(S), key=lambda q: (load[q], q))
        assert slot_of[b] == k
        load[k] += w[b]
    # Longest-processing-time bound: the slots differ by at most the largest job.
    assert max(load) - min(load) <= max(w)


def test_split_batch_plan_fits_free_memory_and_caps(lib):
    ms, ns, ss = _config4_shapes()
    assert orth.split_batch_plan(ms, ns, ss, free_bytes=2 << 30)["slots"] == 1
    few = orth.split_batch_plan(ms, ns, ss, free_bytes=12 << 30)["slots"]
    assert 1 <= few < 16
    assert orth.split_batch_plan(ms, ns, ss, free_bytes=-1)["slots"] == 16      # no memory limit
    one = orth.split_batch_plan(ms, ns, ss, free_bytes=270 << 30, max_slots=1)
    assert one["slots"] == 1 and set(one["slot_of"]) == {0}
    three = orth.split_batch_plan(ms[:3], ns[:3], ss[:3])
    assert three["slots"] == 3 and sorted(three["slot_of"]) == [0, 1, 2]
    assert orth.split_batch_plan([], [], [])["slots"] == 0


def test_split_staged_dry_run_config4():
    """The staged split-precision plan of the config-4 batch (4096 matrices): a few
    hundred launches per wave (not about a hundred per matrix), more waves for a
    smaller budget, and s > 16 refused (the staged form's limit)."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    ms, ns, ss, _ = bench.batch_shapes(4096, 2024)
    big = orth.split_batch_dry_run(ms, ns, ss, 80 << 30)
    small = orth.split_batch_dry_run(ms, ns, ss, 20 << 30)
    assert big["rc"] == 0 and small["rc"] == 0
    assert small["waves"] > big["waves"] >= 2
    for d in (big, small):
        assert d["launches"] / d["waves"] < 250, d
        assert d["bytes"] <= (80 << 30)
    assert orth.split_batch_dry_run([3000], [64], [32], 1 << 30)["rc"] == 4
