"""Benchmark: one BCGSI+P-1S QR of a tall-skinny FP64 matrix on one GB300.

A "step" is one full QR (the reference's bcgsi2P1s, SRC/orth.c:48-222) of the
m x n matrix X = U diag(sigma) W^T (U, W Q factors of seeded Gaussians, sigma
log-spaced from 1 to 1/kappa), m = 2^23, n = 512, s = 16, kappa = 1e6: the
configuration the reference's headline metric is quoted on. Synthetic data of
that construction stands in for any dataset (there is none).

Per step the input is restored from a resident copy (a device-to-device copy
outside the timed interval: the QR overwrites X in place); the QR itself is
timed with CUDA events on the launching stream. X is 34 GB, far larger than the
129 MB L2, so no L2 flush is needed between steps.

Output: one JSON line (rank 0). `value` is ms per QR with X resident in HBM;
`e2e` is the same QR through the orth.h host entry point with host buffers
(host->device and device->host copies inside the timed interval); `roofline`
is the dominant kernel's algorithmic rate against the measured peak of the pipe
that bounds it; `cpu_baseline` times the oracle (the numpy/OpenBLAS restatement
of the reference) on a bounded sample of the same workload on the host cores.

`--impl reference` times the reference's CPU algorithm (the oracle restatement;
the reference's own build cannot run on this host) on the host cores.

Other workloads (not the default line):
  --workload batched [--precision split]   4096 independent matrices of uneven m, s,
      p and kappa in one batched plan (matrices/s, worst-case LOO over the batch);
  --workload sweep [--variant V --kappas ... --block s --monomial]   accuracy and
      time per condition number in FP64 and both split forms.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

# Split-precision batches run up to 16 concurrent streams; give each its own
# hardware work queue (must be set before CUDA starts).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "one-synchronization-bcgs_gb300"))

METRIC = "ms per BCGSI+P-1S QR (m=2^23, n=512, s=16, FP64 in/out, LOO<=1e-12)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--variant", default="bcgsi2P1s")
    ap.add_argument("--m", "--rows", dest="m", type=int, default=1 << 23)
    ap.add_argument("--n", "--cols", dest="n", type=int, default=512)
    ap.add_argument("--s", "--block", dest="s", type=int, default=16)
    ap.add_argument("--kappa", type=float, default=1e6)
    ap.add_argument("--precision", choices=["auto", "fp64", "split"], default="auto")
    ap.add_argument("--fp64-steps", type=int, default=1,
                    help="timed FP64 QRs reported beside a split-precision run")
    ap.add_argument("--fast-steps", type=int, default=1,
                    help="timed 48-bit split QRs reported beside the 56-bit split run")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--e2e-cuda-host-alloc", action="store_true",
                    help="add an e2e leg on cudaHostAlloc host buffers beside the huge-page ones")
    ap.add_argument("--e2e-pageable", action="store_true",
                    help="add an e2e leg on pageable (malloc) host buffers, two samples")
    ap.add_argument("--cpu-rows", type=int, default=1 << 21,
                    help="rows of the bounded CPU sample of the cpu_baseline leg (time scaled to m)")
    ap.add_argument("--ref-budget-s", type=float, default=180.0,
                    help="--impl reference: wall-time budget of the timed full-size steps")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--kappas", default="1e2,1e6,1e10,1e14", help="sweep workload: condition numbers")
    ap.add_argument("--precisions", default="fp64,split7,split6", help="sweep workload: forms to run")
    ap.add_argument("--monomial", action="store_true",
                    help="sweep workload: add the s-step monomial basis (m=2^22, s=8, n=512)")
    ap.add_argument("--workload", choices=["qr", "batched", "sweep"], default="qr",
                    help="qr: one BCGSI+P-1S QR of m x n (default); batched: the batched form "
                         "(--batch matrices of uneven m, s, p and kappa in one captured CUDA graph)")
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--batch-seed", type=int, default=2024)
    ap.add_argument("--no-tune", action="store_true")
    return ap.parse_args()


def max_over_ranks(value: float, world: int, device=None) -> float:
    """The slowest replica's value (all ranks get it); identity for one rank."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak(key: str):
    """A figure from MEASURED_PEAKS.json (written on the GPU machine), or None."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            v = json.load(f).get(key)
        return float(v) if v else None
    except (OSError, ValueError):
        return None


def alg_bytes_p1s(m: int, n: int, s: int) -> float:
    """Algorithmic HBM bytes of one BCGSI+P-1S QR: one read of Q_{1:k-1} per
    block step plus reading X, writing Q and writing+reading U once:
    8 m [s P (P-1)/2 + 4 n] with P = n/s blocks."""
    P = n // s
    return 8.0 * m * (s * P * (P - 1) / 2.0 + 4.0 * n)


def alg_flops_p1s(m: int, n: int, s: int) -> float:
    """Algorithmic flops of one BCGSI+P-1S QR: 4 m n^2 + 8 m n s."""
    return 4.0 * m * n * n + 8.0 * m * n * s


def traffic_ratio(kernel_class: str):
    """ncu DRAM bytes / traffic bytes (the bytes the kernels as built move at
    least) of a kernel class, from the committed ncu summary
    (profiles/traffic.json), or None when no capture of the current kernel has
    been summarized."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    try:
        v = json.load(open(p)).get(kernel_class)
        return float(v) if v is not None else None
    except Exception:
        return None


def host_input(m: int, n: int, kappa: float, seed: int):
    """The bench's input X (m x n, column-major float64) on the host: built on the
    GPU by the same seeded construction as the timed arm when one is present
    (torch only; none of this library's kernels), else by numpy."""
    from bcgs_gb300 import inputs
    try:
        import torch
        if torch.cuda.is_available():
            Xt = inputs.graded_device(m, n, kappa, seed=seed, device="cuda")
            Xh = Xt.cpu().numpy()          # (n, m) row-major == X column-major
            del Xt
            torch.cuda.empty_cache()
            return Xh.T
    except ImportError:
        pass
    return inputs.graded_host(m, n, kappa, seed=seed)


def port_step(variant: str, X0, n: int, s: int, work=None):
    """One QR by the oracle (numpy/OpenBLAS restatement of the reference) on a
    working copy of X0; returns the seconds of the QR itself. The copy into the
    preallocated working buffer is outside the interval, as the reference's own
    driver factors X in place (TESTS/test_orth.c:46-52)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bcgs_port
    m = X0.shape[0]
    ncols = max(n + s, 3 * s)
    if work is None or work.shape != (m, ncols):
        work = np.zeros((m, ncols), order="F")
    work[:, :n] = X0
    R = np.zeros((n, n), order="F")
    t0 = time.perf_counter()
    bcgs_port.VARIANTS[variant](work, n, s, R)
    return time.perf_counter() - t0, work


def cpu_sample(args, rows: int):
    """Time the oracle on the first `rows` rows' worth of the same workload (a
    bounded sample); return seconds and thread count."""
    X = host_input(rows, args.n, args.kappa, seed=1234)
    dt, _ = port_step(args.variant, X, args.n, args.s)
    return dt, os.cpu_count()


def run_reference(args, rank, world):
    """The reference's algorithm on the host cores, at the full workload.

    The reference's own build needs its sources and an x86 OpenBLAS, so the
    oracle restatement (pinned to that build by the tests) runs here with
    OpenBLAS on every host thread. Each timed step is one full-size QR (about
    46 s on 16 Grace cores at m = 2^23), so the steps run are bounded by
    --ref-budget-s: the line reports how many ran. Each warm-up step is one QR of
    a 2^16-row sample (thread pools, first-touch of the library)."""
    if rank != 0:
        return
    m, n, s = args.m, args.n, args.s
    t_gen = time.perf_counter()
    X0 = host_input(m, n, args.kappa, seed=1234)
    t_gen = time.perf_counter() - t_gen
    warm = 0
    if args.warmup > 0:
        Xs = X0[: min(m, 1 << 16), :].copy(order="F")
        for _ in range(args.warmup):
            port_step(args.variant, Xs.copy(order="F"), n, s)
            warm += 1
        del Xs
    steps, work = [], None
    t_start = time.perf_counter()
    for _ in range(max(1, args.steps)):
        dt, work = port_step(args.variant, X0, n, s, work)
        steps.append(dt)
        if time.perf_counter() - t_start + dt > args.ref_budget_s:
            break
    ms = sum(steps) / len(steps) * 1e3
    threads = os.cpu_count()
    sample = (f"{len(steps)} full-size {args.variant} QRs of m={m} x n={n}, s={s} by the numpy/OpenBLAS "
              f"restatement of the reference on {threads} host threads (steps bounded by a "
              f"{args.ref_budget_s:.0f} s budget; each warm-up step: one QR of a 2^16-row sample)")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(ms, 3), "unit": "ms",
        "n_gpus": args.gpus, "steps": len(steps), "steps_requested": args.steps, "warmup": warm,
        "ms_per_step": round(ms, 3), "step_ms": [round(x * 1e3, 1) for x in steps],
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"{args.variant} QR m={m} n={n} s={s} kappa={args.kappa:g} "
                               f"(graded X = U diag(sigma) W^T)", "input_build_s": round(t_gen, 1)},
        "cpu_baseline": {"value": round(ms, 3), "unit": "ms", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(ms, 3), "unit": "ms", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist

    from bcgs_gb300 import inputs, orth

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    orth.load()
    m, n, s = args.m, args.n, args.s
    variant = args.variant
    split_ok = orth.split_supported(m, n, s)
    if args.precision == "fp64" or (args.precision == "auto" and not split_ok):
        prec, prec_name = orth.FP64, "fp64"
    else:
        prec, prec_name = orth.SPLIT_BF16, "split_bf16x7 (56-bit digit planes on tcgen05)"

    def barrier():
        if world > 1:
            dist.barrier()

    X0 = inputs.graded_device(m, n, args.kappa, seed=1234 + rank, device=str(dev))  # (n, m)
    X = torch.empty_like(X0)
    R = torch.zeros((n, n), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    if orth.reserve(m, n, s) != 0:
        raise RuntimeError("workspace reservation failed")

    def one_qr(precision, timed_events=None):
        with torch.cuda.stream(stream):
            X.copy_(X0)
            R.zero_()
            if timed_events is not None:
                timed_events[0].record(stream)
            rc, _ = orth.run_dev(variant, m, n, s, X.data_ptr(), m, R.data_ptr(), n, precision,
                                 sptr, want_status=False)
            if timed_events is not None:
                timed_events[1].record(stream)
        if rc != 0:
            raise RuntimeError(f"run_dev rc={rc}")

    for _ in range(max(0, args.warmup)):
        one_qr(prec)
    torch.cuda.synchronize()
    launches_per_qr = orth.last_launch_count()

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    orth.profile(True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            one_qr(prec, evs[k])
        torch.cuda.synchronize()
    barrier()
    prof = orth.profile_read()
    orth.profile(False)
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms = max_over_ranks(sum(step_ms) / len(step_ms), world, dev)

    # Accuracy of a finished QR: the library's metrics kernels (the reference's
    # test_orth_accuracy on the device; Q^T Q from the exact-accumulation digit Gram,
    # double-double sums), and the 2-norm LOO from the symmetric error matrix.
    def accuracy():
        import numpy as np
        E = torch.empty((n, n), dtype=torch.float64, device=dev)
        gp = orth.SPLIT_BF16 if orth.split_supported(m, n, 16) else orth.FP64
        rc, loo_f, res_f, x_f = orth.accuracy_dev(m, n, X0.data_ptr(), m, X.data_ptr(), m, R.data_ptr(), n,
                                                  gp, E.data_ptr(), n, sptr)
        if rc != 0:
            raise RuntimeError(f"accuracy_dev rc={rc}")
        Eh = E.cpu().numpy()
        return {"loo_2": float(np.max(np.abs(np.linalg.eigvalsh(Eh)))), "loo_fro": loo_f,
                "rel_residual": res_f / x_f if x_f > 0 else 0.0,
                "metric": "orth_gb300_accuracy_dev (exact digit Gram, double-double sums)"}

    acc = {} if args.no_accuracy else accuracy()

    def side_leg(precision, steps):
        one_qr(precision)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        for k in range(steps):
            one_qr(precision, ev[k])
        torch.cuda.synchronize()
        ms_ = sum(a.elapsed_time(b) for a, b in ev) / len(ev)
        return ms_, ({} if args.no_accuracy else accuracy())

    # End to end through the orth.h host entry point (page-locked host buffers), right
    # after the timed region, before the side legs change the GPU's state. The buffers
    # come from the library's orth_gb300_host_alloc (huge-page backed, registered);
    # --e2e-cuda-host-alloc adds a leg on cudaHostAlloc memory (torch pin_memory).
    e2e = None
    if not args.no_e2e and args.e2e_steps > 0:
        import numpy as np

        def host_leg(Xh, Rh, samples):
            Xh_t = torch.from_numpy(Xh.T)      # (n, m) view of the m x n column-major buffer
            Rh_t = torch.from_numpy(Rh.T)
            work = np.zeros(1)
            times, timelines = [], []
            for k in range(samples + 1):
                Xh_t.copy_(X0, non_blocking=False)
                Rh_t.zero_()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                rc = orth.call(variant, m, n, s, Xh, m, Rh, n, work, orth.lwork_min(m, n, s, variant))
                dt = time.perf_counter() - t0
                if rc != 0:
                    raise RuntimeError(f"host entry point rc={rc}")
                if k > 0:   # first call warms the host-path buffers
                    times.append(dt * 1e3)
                    timelines.append(orth.last_host_timing())
            return times, {key: round(sum(t[key] for t in timelines) / len(timelines), 1) for key in timelines[0]}

        orth.set_host_precision(prec)
        try:
            hx, hr = orth.HostBuffer(m * n * 8), orth.HostBuffer(n * n * 8)
            Xh, Rh = hx.array((m, n)), hr.array((n, n))
            kind, huge = hx.info()
            buf_kind = ("page-locked huge-page buffers from orth_gb300_host_alloc" if kind == 1 else
                        "cudaHostAlloc buffers from orth_gb300_host_alloc (huge pages unavailable)")
            host_buf = {"kind": "huge-page mapping" if kind == 1 else "cudaHostAlloc",
                        "x_bytes_on_huge_pages": huge, "x_bytes": m * n * 8}
        except RuntimeError:
            # Several ranks on one host may not get that much page-locked memory:
            # the CUDA allocator's page-locked buffers instead.
            hx = hr = None
            Xh = torch.empty((n, m), dtype=torch.float64, pin_memory=True).numpy().T
            Rh = torch.zeros((n, n), dtype=torch.float64, pin_memory=True).numpy().T
            buf_kind = "cudaHostAlloc buffers (orth_gb300_host_alloc failed)"
            host_buf = {"kind": "torch pin_memory"}
        times, timeline = host_leg(Xh, Rh, args.e2e_steps)
        del Xh, Rh
        if hx is not None:
            hx.close()
            hr.close()
        e2e_ms = max_over_ranks(sum(times) / len(times), world, dev)
        e2e = {"value": round(e2e_ms, 3), "unit": "ms", "samples_ms": [round(x, 1) for x in times],
               "timeline_ms": timeline,
               "h2d_bytes_per_step": m * n * 8, "d2h_bytes_per_step": m * n * 8 + n * n * 8,
               "path": f"orth.h {variant} (host pointers: {buf_kind}), {prec_name}", "host_buffer": host_buf}
        if args.e2e_cuda_host_alloc:
            Xc = torch.empty((n, m), dtype=torch.float64, pin_memory=True)
            Rc = torch.zeros((n, n), dtype=torch.float64, pin_memory=True)
            t2, tl2 = host_leg(Xc.numpy().T, Rc.numpy().T, args.e2e_steps)
            e2e["cuda_host_alloc"] = {"value": round(sum(t2) / len(t2), 3), "samples_ms": [round(x, 1) for x in t2],
                                      "timeline_ms": tl2,
                                      "path": "the same call on cudaHostAlloc buffers (torch pin_memory)"}
            del Xc, Rc
        if args.e2e_pageable:
            # Pageable memory from the C library's malloc, as the reference's own
            # driver allocates Xsub (numpy would advise huge pages on its arrays).
            import ctypes
            libc = ctypes.CDLL(None)
            libc.malloc.restype = ctypes.c_void_p
            libc.malloc.argtypes = [ctypes.c_size_t]
            libc.free.argtypes = [ctypes.c_void_p]
            px, pr = libc.malloc(m * n * 8), libc.malloc(n * n * 8)
            if not px or not pr:
                raise RuntimeError("malloc failed")
            Xq = np.ctypeslib.as_array((ctypes.c_double * (m * n)).from_address(px)).reshape((m, n), order="F")
            Rq = np.ctypeslib.as_array((ctypes.c_double * (n * n)).from_address(pr)).reshape((n, n), order="F")
            t3, tl3 = host_leg(Xq, Rq, 2)
            e2e["pageable"] = {"value": round(sum(t3) / len(t3), 3), "samples_ms": [round(x, 1) for x in t3],
                               "timeline_ms": tl3, "path": "the same call on malloc'd (pageable) buffers"}
            del Xq, Rq
            libc.free(px)
            libc.free(pr)

    # FP64 leg and 48-bit split leg beside the 56-bit split run.
    fp64_ms = fp64_acc = fast_ms = fast_acc = None
    if prec != orth.FP64 and args.fp64_steps > 0:
        fp64_ms, fp64_acc = side_leg(orth.FP64, args.fp64_steps)
    if prec != orth.FP64 and args.fast_steps > 0:
        fast_ms, fast_acc = side_leg(orth.SPLIT_BF16_FAST, args.fast_steps)

    # Roofline of the dominant kernel class, on algorithmic bytes (or flops).
    bytes_alg = alg_bytes_p1s(m, n, s)
    flops_alg = alg_flops_p1s(m, n, s)
    dom = max(("gram", "update"), key=lambda c: prof[c]["ms"])
    pc = prof[dom]
    calls = max(1, pc["calls"])
    launch_ms = pc["ms"] / calls
    if prec == orth.FP64:
        peak = orth.fp64_peak_tflops()
        achieved = pc["flops"] / (pc["ms"] * 1e-3) / 1e12 if pc["ms"] > 0 else 0.0
        roof = {"bound": "fp64", "achieved": round(achieved, 4), "peak": round(peak, 4),
                "unit": "TFLOP/s", "frac": round(achieved / peak, 4) if peak else None,
                "traffic": None, "kernel": dom,
                "peak_source": "live DFMA probe (orth_gb300_fp64_peak_probe); MEASURED_PEAKS.json has no FP64 figure",
                "launch_ms": round(launch_ms, 4),
                "flops_per_launch": round(pc["flops"] / calls),
                "whole_qr": {"achieved": round(flops_alg / (ms * 1e-3) / 1e12, 4), "unit": "TFLOP/s",
                             "frac": round(flops_alg / (ms * 1e-3) / 1e12 / peak, 4) if peak else None}}
    else:
        peak = measured_peak("hbm_gbs")
        peak_src = "MEASURED_PEAKS.json hbm_gbs (of measured)"
        if peak is None:
            peak, peak_src = 6800.0, "fallback 6.8 TB/s (of fallback)"
        secs = pc["ms"] * 1e-3
        achieved = pc["bytes"] / secs / 1e9 if secs > 0 else 0.0
        rate = pc["traffic"] / secs / 1e9 if secs > 0 else 0.0
        kd = 7
        tensor_tflops = pc["flops"] * kd * (kd + 1) / 2 / secs / 1e12 if secs > 0 else 0.0
        ratio = traffic_ratio(dom)
        bf16 = measured_peak("bf16_tflops") or 1900.0
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4),
                "traffic": round(ratio * pc["traffic"] / calls) if ratio is not None else None,
                "kernel": {"gram": "gram_tc_kernel<7> + gram_reduce",
                           "update": "bbuild_fused + bdigit + update_tc_kernel<32,7> (fused Q_k/U_k+1 pass)"}[dom],
                "peak_source": peak_src,
                "launch_ms": round(launch_ms, 4),
                "bytes_per_launch": round(pc["bytes"] / calls),
                "bytes_note": "algorithmic: 8 B per element of each operand column read once and each column "
                              "written (FP64-equivalent), per launch of the class's primitive",
                "traffic_rate": {"value": round(rate, 1), "unit": "GB/s", "frac": round(rate / peak, 4),
                                 "bytes_per_launch": round(pc["traffic"] / calls),
                                 "note": "the bytes the kernels as built move: 14 B per element of the BF16 "
                                         "digit planes read, 8 B per FP64 element written"},
                "traffic_note": "DRAM bytes per launch = ncu dram bytes / traffic bytes (profiles/traffic.json) "
                                "x traffic bytes per launch",
                "tensor_tflops_bf16": round(tensor_tflops, 1),
                "tensor_frac_of_bf16_peak": round(tensor_tflops / bf16, 4),
                "whole_qr": {"achieved": round(bytes_alg / (ms * 1e-3) / 1e9, 1), "unit": "GB/s",
                             "frac": round(bytes_alg / (ms * 1e-3) / 1e9 / peak, 4),
                             "bytes": bytes_alg,
                             "note": "8 m [s P (P-1)/2 + 4 n] per BCGSI+P-1S QR"}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        dt, threads = cpu_sample(args, args.cpu_rows)
        cpu = {"value": round(dt * m / args.cpu_rows * 1e3, 3), "unit": "ms", "cores": threads,
               "kind": "port",
               "sample": f"{variant} on {args.cpu_rows} rows x n={n}, s={s} with the numpy/OpenBLAS "
                         f"restatement of the reference; time scaled by m/{args.cpu_rows}"}

    line = {
        "metric": METRIC, "value": round(ms, 3), "unit": "ms", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"{variant} QR m={m} n={n} s={s} kappa={args.kappa:g} "
                               f"(graded X = U diag(sigma) W^T)",
                   "precision": prec_name, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs (34 GB) larger than L2; no flush",
                   "restore": "X restored from a resident copy before each step, outside the timed interval"},
        "hbm_gbs_alg": round(bytes_alg / (ms * 1e-3) / 1e9, 2),
        "tflops_alg": round(flops_alg / (ms * 1e-3) / 1e12, 4),
        "fp64_ms": round(fp64_ms, 3) if fp64_ms is not None else (round(ms, 3) if prec == orth.FP64 else None),
        "accuracy": acc,
        "fp64_accuracy": fp64_acc,
        "split_fast_ms": round(fast_ms, 3) if fast_ms is not None else None,
        "split_fast_accuracy": fast_acc,
        "speedup_vs_fp64_gpu": round(fp64_ms / ms, 2) if fp64_ms else None,
        "gpu_launches": int(launches_per_qr * args.steps),
        "kernel_profile": {k: {"ms": round(v["ms"], 3), "launches": v["launches"], "calls": v["calls"]}
                           for k, v in prof.items()},
        "roofline": roof,
        "clocks": clk.summary(),
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def batch_shapes(count: int, seed: int):
    """The batched workload: m log-uniform in [2e3, 2e5], s in {4, 8, 16}, p uniform
    in [2, 16], kappa log-uniform in [1e2, 1e10], all from one seed (n = s p)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    ms = np.exp(rng.uniform(np.log(2000), np.log(200000), count)).astype(np.int64)
    ss = rng.choice([4, 8, 16], count)
    ps = rng.integers(2, 17, count)
    ks = np.exp(rng.uniform(np.log(1e2), np.log(1e10), count))
    return [int(x) for x in ms], [int(s * p) for s, p in zip(ss, ps)], [int(x) for x in ss], [float(k) for k in ks]


def run_batched(args, rank, world, local_rank):
    """Batched BCGSI+P-1S: the whole batch as one captured CUDA graph per step."""
    import numpy as np
    import torch

    from bcgs_gb300 import inputs, orth

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    orth.load()
    ms, ns, ss, ks = batch_shapes(args.batch, args.batch_seed + rank)
    free, _ = torch.cuda.mem_get_info(dev)
    sizes = [m * n for m, n in zip(ms, ns)]
    # Two copies of the batch (a resident pristine copy and the working one), the
    # R factors and the plan's workspace must fit.
    count = len(ms)
    while count > 1 and 2 * 8 * sum(sizes[:count]) + 8 * sum(n * n for n in ns[:count]) + (32 << 30) > free:
        count = int(count * 0.9)
    ms, ns, ss, ks, sizes = ms[:count], ns[:count], ss[:count], ks[:count], sizes[:count]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    roffs = np.concatenate([[0], np.cumsum([n * n for n in ns])]).astype(np.int64)
    X0 = torch.empty(int(offs[-1]), dtype=torch.float64, device=dev)
    t_gen = time.perf_counter()
    for b in range(count):
        X0[int(offs[b]):int(offs[b + 1])].copy_(
            inputs.graded_device(ms[b], ns[b], ks[b], seed=args.batch_seed * 100003 + b, device=str(dev)).reshape(-1))
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t_gen
    X = X0.clone()
    R = torch.zeros(int(roffs[-1]), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    xp = [X.data_ptr() + 8 * int(o) for o in offs[:-1]]
    rp = [R.data_ptr() + 8 * int(o) for o in roffs[:-1]]
    t_plan = time.perf_counter()
    bprec = orth.SPLIT_BF16 if args.precision == "split" else orth.FP64
    plan = orth.Batch(ms, ns, ss, xp, rp, precision=bprec, tune=not args.no_tune, stream=sptr)
    if plan.rc != 0:
        raise RuntimeError(f"batch plan rc={plan.rc}")
    torch.cuda.synchronize()
    t_plan = time.perf_counter() - t_plan
    info = plan.info()

    def one(ev=None):
        with torch.cuda.stream(stream):
            X.copy_(X0)
            R.zero_()
            if ev is not None:
                ev[0].record(stream)
            if plan.run(sptr) != 0:
                raise RuntimeError("batch run failed")
            if ev is not None:
                ev[1].record(stream)

    for _ in range(max(0, args.warmup)):
        one()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            one(evs[k])
        torch.cuda.synchronize()
    ms_run = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs) / args.steps, world, dev)
    info = plan.info()   # launches per run are known once a run has been enqueued
    _, steps_bd, _, nbroken = plan.status()
    total = count * world
    value = total / (ms_run * 1e-3)

    # Worst-case accuracy over the batch (the library's metrics kernels).
    acc = {}
    if not args.no_accuracy:
        worst_loo, worst_res, worst_b = 0.0, 0.0, -1
        for b in range(count):
            if steps_bd[b] != 0:
                continue   # a reported breakdown: its Q is not a result
            m, n = ms[b], ns[b]
            E = torch.empty((n, n), dtype=torch.float64, device=dev)
            x0 = X0[int(offs[b]):int(offs[b + 1])]
            gp = orth.SPLIT_BF16 if orth.split_supported(m, n, 16) else orth.FP64
            rc, loo_f, res_f, x_f = orth.accuracy_dev(m, n, x0.data_ptr(), m, xp[b], m, rp[b], n, gp,
                                                      E.data_ptr(), n, sptr)
            if rc != 0:
                raise RuntimeError(f"accuracy_dev rc={rc}")
            Eh = E.cpu().numpy()
            loo2 = float(np.max(np.abs(np.linalg.eigvalsh(Eh)))) if np.isfinite(Eh).all() else float("inf")
            if loo2 > worst_loo:
                worst_loo, worst_b = loo2, b
            worst_res = max(worst_res, res_f / x_f)
        acc = {"worst_loo_2": worst_loo, "worst_loo_matrix": {"m": ms[worst_b], "n": ns[worst_b],
                                                               "s": ss[worst_b], "kappa": ks[worst_b]},
               "worst_rel_residual": worst_res, "breakdowns": nbroken,
               "metric": "orth_gb300_accuracy_dev per matrix (exact digit Gram, double-double sums)"}

    flops = sum(4.0 * m * n * n + 8.0 * m * n * s for m, n, s in zip(ms, ns, ss))
    if bprec == orth.FP64:
        peak = orth.fp64_peak_tflops()
        achieved = flops / (ms_run * 1e-3) / 1e12
        roof = {"bound": "fp64_pipe", "achieved": round(achieved, 4), "peak": round(peak, 4), "unit": "TFLOP/s",
                "frac": round(achieved / peak, 4), "traffic": None,
                "note": "whole batch: algorithmic FLOPs (4mn^2 + 8mns per matrix) / graph time; "
                        "peak = DFMA-loop probe"}
    else:
        hbm = measured_peak("hbm_gbs") or 6668.9
        byts = sum(alg_bytes_p1s(m, n, s) for m, n, s in zip(ms, ns, ss))
        achieved = byts / (ms_run * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "traffic": None,
                "note": "whole batch: algorithmic FP64 bytes 8m[sP(P-1)/2 + 4n] per matrix / run time; "
                        "staged tensor-core plan (one launch per stage over each wave's matrices)",
                "tflops_fp64_equivalent": round(flops / (ms_run * 1e-3) / 1e12, 3)}
    cpu = None
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import bcgs_port
        sample = list(range(0, count, max(1, count // 6)))[:6]
        t0 = time.perf_counter()
        for b in sample:
            Xh = inputs.graded_host(ms[b], ns[b], ks[b], seed=b)
            bcgs_port.run_variant("bcgsi2P1s", Xh, ns[b], ss[b])
        dt = time.perf_counter() - t0
        work = sum(sizes[b] * ns[b] for b in sample) / sum(sz * n for sz, n in zip(sizes, ns))
        # The sample holds `work` of the batch's m n^2 work: the whole batch would take dt / work.
        cpu = {"value": round(count / (dt / work), 3), "unit": "matrices/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{len(sample)} matrices of the batch through the oracle (numpy/OpenBLAS), time scaled "
                         f"by the batch's m n^2 work"}
    line = {
        "metric": "matrices/s, batched BCGSI+P-1S (4096 X of m in [2e3,2e5], s in {4,8,16}, p in [2,16], "
                  "kappa in [1e2,1e10])",
        "value": round(value, 3), "unit": "matrices/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_run, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": (f"batched bcgsi2P1s, {count} matrices (seed {args.batch_seed}), FP64, "
                                f"one CUDA graph of {info['launches']} launches per step") if bprec == orth.FP64 else
                               (f"batched bcgsi2P1s, {count} matrices (seed {args.batch_seed}), split_bf16x7, "
                                f"staged: waves of matrices, one launch per stage over a wave, one captured CUDA "
                                f"graph per wave ({info['launches']} launches per step)"),
                   "batch": count, "batch_requested": args.batch, "elements": int(offs[-1]),
                   "tuned_panel_rows": {str(k): v for k, v in info["tuned"].items()},
                   "l2": f"inputs ({8 * int(offs[-1]) / 1e9:.0f} GB) larger than L2; no flush",
                   "restore": "X restored from a resident copy before each step, outside the timed interval",
                   "setup_s": {"generate": round(t_gen, 1), "plan_tune_capture": round(t_plan, 2)}},
        "accuracy": acc,
        "gpu_launches": int(info["launches"] * args.steps),
        "roofline": roof,
        "clocks": clk.summary(),
        "e2e": None,
        "e2e_note": "the batch is 120 GB; a pinned host copy of it is not held, so no host-buffer run",
        "cpu_baseline": cpu,
    }
    plan.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_sweep(args, rank, world, local_rank):
    """Accuracy and time per condition number (and for the monomial basis): the
    variant in FP64 and both split-precision forms, with the library's metrics."""
    import numpy as np
    import torch

    from bcgs_gb300 import inputs, orth

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    orth.load()
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    cases = [("graded", float(k), args.m, args.n, args.s) for k in args.kappas.split(",") if k]
    if args.monomial:
        cases.append(("monomial", None, 1 << 22, 512, 8))
    rows = []
    for kind, kappa, m, n, s in cases:
        if kind == "graded":
            X0 = inputs.graded_device(m, n, kappa, seed=1234, device=str(dev))
        else:
            X0 = inputs.monomial_device(m, n, s, seed=1234, device=str(dev))
        X = torch.empty_like(X0)
        R = torch.zeros((n, n), dtype=torch.float64, device=dev)
        E = torch.empty((n, n), dtype=torch.float64, device=dev)
        precs = [("fp64", orth.FP64)]
        if orth.split_supported(m, n, s):
            precs += [("split7", orth.SPLIT_BF16), ("split6", orth.SPLIT_BF16_FAST)]
        precs = [pr for pr in precs if pr[0] in args.precisions.split(",")]
        for name, prec in precs:
            times, st = [], None
            for k in range(2):
                with torch.cuda.stream(stream):
                    X.copy_(X0)
                    R.zero_()
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    rc, st = orth.run_dev(args.variant, m, n, s, X.data_ptr(), m, R.data_ptr(), n, prec, sptr)
                    b.record(stream)
                if rc != 0:
                    raise RuntimeError(f"run_dev rc={rc}")
                torch.cuda.synchronize()
                if k > 0:
                    times.append(a.elapsed_time(b))
            gp = orth.SPLIT_BF16 if orth.split_supported(m, n, 16) else orth.FP64
            rc, loo_f, res_f, x_f = orth.accuracy_dev(m, n, X0.data_ptr(), m, X.data_ptr(), m, R.data_ptr(), n, gp,
                                                      E.data_ptr(), n, sptr)
            if rc != 0:
                raise RuntimeError(f"accuracy_dev rc={rc}")
            Eh = E.cpu().numpy()
            finite = bool(np.isfinite(Eh).all())
            rows.append({"input": kind, "kappa": kappa, "m": m, "n": n, "s": s, "precision": name,
                         "ms": round(times[0], 3),
                         "loo_2": float(np.max(np.abs(np.linalg.eigvalsh(Eh)))) if finite else None,
                         "loo_fro": loo_f, "rel_residual": res_f / x_f if x_f > 0 else 0.0,
                         "breakdown_step": st["breakdown_step"], "breakdown_info": st["breakdown_info"]})
            print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
        del X0, X
        torch.cuda.empty_cache()
    if rank == 0:
        print(json.dumps({"metric": "accuracy and ms per QR across condition numbers", "variant": args.variant,
                          "workload": "sweep", "metrics": "orth_gb300_accuracy_dev (exact digit Gram)",
                          "rows": rows}), flush=True)


def main():
    args = parse()
    rank, world, local_rank = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.gpus > 1 else "gloo")
    try:
        if args.workload == "batched":
            run_batched(args, rank, world, local_rank)
        elif args.workload == "sweep":
            run_sweep(args, rank, world, local_rank)
        else:
            run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
