"""CPU tests of the row-sharded path's host side (no GPU).

* orth_gb300_shard_rows follows the reference's 1-D block-row partition
  (SRC/orth.c:69-76, TESTS/test_orth.c:24-32) at the granularity of
  ORTH_GB300_SHARD_ROWS-row chunks: contiguous, covering, the extra chunks on
  the last ranks.
* The exchange protocol, on two gloo ranks (world size 2, 127.0.0.1): each rank
  forms the per-chunk partial Gram sums of its rows, pads them to the largest
  chunk count with zeros, gathers every rank's block in rank order, and sums the
  chunks in global order. The sum is bit-identical to one rank's sum over the
  same chunks. (The CUDA kernels do the partial sums on the GPU; numpy stands in
  for them here.)
"""
import os

import numpy as np
import pytest

from bcgs_gb300 import orth

ROWS = orth.SHARD_ROWS


@pytest.mark.parametrize("m", [8192, 8193, 100000, 3 * 8192 + 1234, 1 << 20])
def test_shard_rows_partition(lib, m):
    nch = -(-m // ROWS)
    for size in range(1, 9):
        if size > nch:
            with pytest.raises(ValueError):
                orth.shard_rows(m, size, 0)
            continue
        parts = [orth.shard_rows(m, size, r) for r in range(size)]
        assert parts[0][0] == 0 and sum(ms for _, ms in parts) == m
        for r in range(size - 1):
            assert parts[r][0] + parts[r][1] == parts[r + 1][0]
            assert parts[r][1] % ROWS == 0
        counts = [-(-ms // ROWS) for _, ms in parts]
        cpr, res = nch // size, nch % size
        assert counts == [cpr + (1 if r >= size - res else 0) for r in range(size)]


def _worker(rank, size, port, m, n, out):
    import torch.distributed as dist
    import torch
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=size)
    from bcgs_gb300 import orth as o
    rng = np.random.default_rng(5)
    X = rng.standard_normal((m, n))
    r0, ms = o.shard_rows(m, size, rank)
    nch = -(-ms // ROWS)
    maxc = max(-(-o.shard_rows(m, size, r)[1] // ROWS) for r in range(size))
    part = np.zeros((maxc, n, n))
    for c in range(nch):
        Xc = X[r0 + c * ROWS: r0 + min(ms, (c + 1) * ROWS)]
        part[c] = Xc.T @ Xc
    t = torch.from_numpy(part.reshape(-1))
    outs = [torch.empty_like(t) for _ in range(size)]
    dist.all_gather(outs, t)
    allp = np.concatenate([x.numpy() for x in outs]).reshape(size * maxc, n, n)
    G = np.zeros((n, n))
    for c in range(size * maxc):
        G = G + allp[c]
    np.save(out, G)
    dist.destroy_process_group()


def test_exchange_protocol_two_gloo_ranks(tmp_path):
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    m, n = 2 * ROWS + 777, 6          # 3 chunks: rank 0 holds 1 (padded to 2), rank 1 holds 2
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_worker, args=(r, 2, port, m, n, str(tmp_path / f"g{r}.npy"))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    G0, G1 = np.load(tmp_path / "g0.npy"), np.load(tmp_path / "g1.npy")
    # One rank: the same chunks, summed in the same order.
    X = np.random.default_rng(5).standard_normal((m, n))
    G = np.zeros((n, n))
    for c in range(-(-m // ROWS)):
        Xc = X[c * ROWS:(c + 1) * ROWS]
        G = G + Xc.T @ Xc
    assert np.array_equal(G0, G) and np.array_equal(G1, G)
