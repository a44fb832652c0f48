"""One rank of a row-sharded QR, run as its own process (launched by
tests/test_sharded_gpu.py with RANK, WORLD_SIZE, MASTER_ADDR, MASTER_PORT set).

The rank builds the seeded input, takes its rows by orth_gb300_shard_rows, and
runs orth_gb300_run_sharded for each requested variant with a host-staged
allgather over a gloo process group (world size 1: no process group). It writes
its rows of Q, R, the status and the reduction count to an .npz file.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "one-synchronization-bcgs_gb300"))


def main(out_path, m, n, s, variants):
    import torch
    import torch.distributed as dist

    from bcgs_gb300 import inputs, orth
    rank, size = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    if size > 1:
        dist.init_process_group("gloo", rank=rank, world_size=size)

    def gather_host(a):
        if size == 1:
            return [a]
        t = torch.from_numpy(a)
        outs = [torch.empty_like(t) for _ in range(size)]
        dist.all_gather(outs, t)
        return [o.numpy() for o in outs]

    cb = orth.host_staged_allgather(gather_host)
    X = inputs.graded_host(m, n, 1e6, seed=17)
    r0, ms = orth.shard_rows(m, size, rank)
    stream = torch.cuda.current_stream().cuda_stream
    res = {"row0": np.array(r0), "msub": np.array(ms)}
    for v in variants:
        dX = torch.from_numpy(np.ascontiguousarray(X[r0:r0 + ms].T)).cuda()   # (n, msub) == rows, column-major
        dR = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        rc, st = orth.run_sharded(v, m, n, s, dX.data_ptr(), ms, dR.data_ptr(), n, rank, size, cb, stream)
        res[f"{v}/rc"] = np.array(rc)
        res[f"{v}/step"] = np.array(st["breakdown_step"])
        res[f"{v}/reductions"] = np.array(orth.last_reduction_count())
        res[f"{v}/Q"] = dX.cpu().numpy().T.copy()
        res[f"{v}/R"] = dR.cpu().numpy().T.copy()
    np.savez(out_path, **res)
    if size > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main(sys.argv[1], int(sys.argv[2]), int(sys.argv[3]), int(sys.argv[4]), sys.argv[5].split(","))
