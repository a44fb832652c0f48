"""Python binding of the GB300 BCGS C ABI (include/orth.h, include/orth_gb300.h).

The five reference entry points keep their names and argument meanings
(reference include/orth.h:8-17); they take numpy float64 arrays in Fortran order
and call straight into ``liborth_gb300.so``. There is no fallback: if the
library is missing or cannot load, every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

VARIANTS = ("bcgsi2P1s", "bcgsi21s", "bcgspipi2", "bcgsi2", "bcgsi2P2s")
VARIANT_ID = {name: i for i, name in enumerate(VARIANTS)}
FP64 = 0
SPLIT_BF16 = 1          # 7 BF16 digit planes (56-bit fixed point)
SPLIT_BF16_FAST = 2     # 6 BF16 digit planes (48-bit fixed point)


class Status(ctypes.Structure):
    _fields_ = [("breakdown_step", ctypes.c_int), ("breakdown_info", ctypes.c_int),
                ("timeout", ctypes.c_int), ("cuda_error", ctypes.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


ALLGATHER_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_longlong, ctypes.c_void_p)


class Comm(ctypes.Structure):
    """orth_gb300_comm: this rank, the rank count and the allgather callback."""
    _fields_ = [("rank", ctypes.c_int), ("size", ctypes.c_int), ("allgather", ALLGATHER_FN),
                ("ctx", ctypes.c_void_p)]


_lib = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(path: str | None = None):
    """Load (once) and return the ctypes handle of liborth_gb300.so."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or _build.LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"liborth_gb300.so not built ({p}); run bcgs_gb300.build.build()")
    lib = ctypes.CDLL(p)
    dp = ctypes.POINTER(ctypes.c_double)
    for name in VARIANTS:
        f = getattr(lib, name)
        f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, dp, ctypes.c_int,
                      dp, ctypes.c_int]
        f.restype = ctypes.c_int
    lib.orth_gb300_run_dev.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.POINTER(Status)]
    lib.orth_gb300_run_dev.restype = ctypes.c_int
    lib.orth_gb300_last_status.argtypes = [ctypes.POINTER(Status)]
    lib.orth_gb300_last_status.restype = None
    lib.orth_gb300_last_host_timing.argtypes = [ctypes.POINTER(ctypes.c_double)]
    lib.orth_gb300_last_host_timing.restype = None
    lib.orth_gb300_sync_count.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.orth_gb300_sync_count.restype = ctypes.c_int
    lib.orth_gb300_last_launch_count.argtypes = []
    lib.orth_gb300_last_launch_count.restype = ctypes.c_longlong
    lib.orth_gb300_last_reduction_count.argtypes = []
    lib.orth_gb300_last_reduction_count.restype = ctypes.c_longlong
    lib.orth_gb300_profile.argtypes = [ctypes.c_int]
    lib.orth_gb300_profile.restype = None
    lib.orth_gb300_profile_read.argtypes = [ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_longlong),
                                            ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_double)]
    lib.orth_gb300_profile_read.restype = ctypes.c_int
    lib.orth_gb300_profile_traffic.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]
    lib.orth_gb300_profile_traffic.restype = ctypes.c_int
    lib.orth_gb300_fp64_peak_probe.argtypes = [ctypes.POINTER(ctypes.c_double)]
    lib.orth_gb300_fp64_peak_probe.restype = ctypes.c_int
    lib.orth_gb300_bcgsi2P1s_dev_noalloc.argtypes = [
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong,
        ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(Status)]
    lib.orth_gb300_bcgsi2P1s_dev_noalloc.restype = ctypes.c_int
    lib.orth_gb300_shard_rows.argtypes = [ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
    lib.orth_gb300_shard_rows.restype = ctypes.c_int
    lib.orth_gb300_run_sharded.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.POINTER(Comm), ctypes.POINTER(Status)]
    lib.orth_gb300_run_sharded.restype = ctypes.c_int
    lib.orth_gb300_set_intra_ortho.argtypes = [ctypes.c_int]
    lib.orth_gb300_set_intra_ortho.restype = ctypes.c_int
    lib.orth_gb300_set_host_precision.argtypes = [ctypes.c_int]
    lib.orth_gb300_set_host_precision.restype = ctypes.c_int
    lib.orth_gb300_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]
    lib.orth_gb300_host_alloc.restype = ctypes.c_int
    lib.orth_gb300_host_free.argtypes = [ctypes.c_void_p]
    lib.orth_gb300_host_free.restype = ctypes.c_int
    lib.orth_gb300_host_buffer_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                                ctypes.POINTER(ctypes.c_longlong)]
    lib.orth_gb300_host_buffer_info.restype = ctypes.c_int
    lib.orth_gb300_last_split_error.argtypes = []
    lib.orth_gb300_last_split_error.restype = ctypes.c_int
    lib.orth_gb300_split_supported.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.orth_gb300_split_supported.restype = ctypes.c_int
    lib.orth_gb300_gram_dev.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.orth_gb300_gram_dev.restype = ctypes.c_int
    lib.orth_gb300_accuracy_dev.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong,
                                            ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                            ctypes.POINTER(ctypes.c_double)]
    lib.orth_gb300_accuracy_dev.restype = ctypes.c_int
    lib.orth_gb300_set_gram_chunk_rows.argtypes = [ctypes.c_longlong]
    lib.orth_gb300_split_slice_dev.argtypes = [ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong,
                                               ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.orth_gb300_split_slice_dev.restype = ctypes.c_int
    lib.orth_gb300_poison_shared_memory.argtypes = [ctypes.c_ulonglong, ctypes.c_void_p]
    lib.orth_gb300_poison_shared_memory.restype = ctypes.c_int
    lib.orth_gb300_timeout_probe.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
    lib.orth_gb300_timeout_probe.restype = ctypes.c_int
    lib.orth_gb300_set_gram_chunk_rows.restype = None
    P_int, P_ll, P_vp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_void_p)
    lib.orth_gb300_batch_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, P_int, P_int,
                                            P_int, P_vp, P_ll, P_vp, P_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_void_p]
    lib.orth_gb300_batch_create.restype = ctypes.c_int
    lib.orth_gb300_batch_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.orth_gb300_batch_run.restype = ctypes.c_int
    lib.orth_gb300_batch_status.argtypes = [ctypes.c_void_p, P_int, P_int, P_int]
    lib.orth_gb300_batch_status.restype = ctypes.c_int
    lib.orth_gb300_batch_info.argtypes = [ctypes.c_void_p, P_ll, P_ll, P_int, P_int]
    lib.orth_gb300_batch_info.restype = ctypes.c_int
    lib.orth_gb300_batch_destroy.argtypes = [ctypes.c_void_p]
    lib.orth_gb300_batch_destroy.restype = None
    lib.orth_gb300_batch_dry_run.argtypes = [ctypes.c_int, P_int, P_int, P_int, P_ll, P_ll, P_ll]
    lib.orth_gb300_batch_dry_run.restype = ctypes.c_int
    lib.orth_gb300_split_batch_dry_run.argtypes = [ctypes.c_int, P_int, P_int, P_int, ctypes.c_longlong, P_int, P_ll,
                                                   P_ll]
    lib.orth_gb300_split_batch_dry_run.restype = ctypes.c_int
    lib.orth_gb300_split_batch_plan.argtypes = [ctypes.c_int, P_int, P_int, P_int, ctypes.c_longlong, ctypes.c_int,
                                                P_int, P_int]
    lib.orth_gb300_split_batch_plan.restype = ctypes.c_int
    lib.orth_gb300_reserve.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.orth_gb300_reserve.restype = ctypes.c_int
    lib.orth_gb300_release.argtypes = []
    lib.orth_gb300_release.restype = None
    lib.orth_gb300_version.argtypes = []
    lib.orth_gb300_version.restype = ctypes.c_char_p
    _lib = lib
    return lib


def lwork_min(m: int, n: int, s: int, variant: str = "bcgsi2P1s") -> int:
    """The reference's minimum lwork (SRC/orth.c:82, :489 for bcgsi2)."""
    tall = m * s if variant == "bcgsi2" else m * n
    return min(5 * n * s + 9 * s * s + tall, 2**31 - 1)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def call(variant: str, m: int, n: int, s: int, Xsub: np.ndarray, ldXsub: int, R: np.ndarray,
         ldR: int, work: np.ndarray | None = None, lwork: int | None = None) -> int:
    """Call the orth.h entry point ``variant`` exactly as C code would."""
    lib = load()
    if Xsub.dtype != np.float64 or R.dtype != np.float64:
        raise TypeError("Xsub and R must be float64")
    if lwork is None:
        lwork = lwork_min(m, n, s, variant)
    if work is None:
        work = np.zeros(1)
    return int(getattr(lib, variant)(m, n, s, _dp(Xsub), ldXsub, _dp(R), ldR, _dp(work), lwork))


def call_ptr(variant: str, m: int, n: int, s: int, x_ptr: int, ldXsub: int, r_ptr: int, ldR: int,
             lwork: int | None = None) -> int:
    """Call the orth.h entry point ``variant`` with raw addresses (host or device
    memory, e.g. ``tensor.data_ptr()``), as C code holding such pointers would."""
    lib = load()
    if lwork is None:
        lwork = lwork_min(m, n, s, variant)
    dp = ctypes.POINTER(ctypes.c_double)
    work = np.zeros(1)
    return int(getattr(lib, variant)(m, n, s, ctypes.cast(ctypes.c_void_p(x_ptr), dp), ldXsub,
                                     ctypes.cast(ctypes.c_void_p(r_ptr), dp), ldR, _dp(work), lwork))


def qr(variant: str, X0: np.ndarray, s: int):
    """Convenience: QR of a copy of X0 (m x n) through the orth.h entry point.

    Returns (Q, R, rc, status_dict)."""
    m, n = X0.shape
    X = np.array(X0, dtype=np.float64, order="F", copy=True)
    R = np.zeros((n, n), order="F")
    rc = call(variant, m, n, s, X, m, R, n)
    return X, R, rc, last_status()


def last_status() -> dict:
    st = Status()
    load().orth_gb300_last_status(ctypes.byref(st))
    return st.as_dict()


def timeout_probe(code: int, stream: int = 0):
    """Makes one bounded device wait run out (orth_gb300_timeout_probe): returns
    (rc, recorded code, abort flag)."""
    out = (ctypes.c_int * 2)()
    rc = int(load().orth_gb300_timeout_probe(code, ctypes.c_void_p(stream), out))
    return rc, out[0], out[1]


class HostBuffer:
    """Page-locked, huge-page-backed host memory from orth_gb300_host_alloc.

    ``array(shape, order)`` gives a float64 numpy view of it (zero-filled at
    allocation). The buffer is released by ``close()`` or when the object is
    collected; views must not outlive it.
    """

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        self._p = ctypes.c_void_p(0)
        rc = int(load().orth_gb300_host_alloc(ctypes.c_size_t(self.nbytes), ctypes.byref(self._p)))
        if rc != 0:
            raise RuntimeError(f"orth_gb300_host_alloc({self.nbytes}) returned {rc}")

    @property
    def ptr(self) -> int:
        return int(self._p.value or 0)

    def array(self, shape, order: str = "F"):
        import numpy as np
        count = int(np.prod(shape))
        if count * 8 > self.nbytes:
            raise ValueError("shape exceeds the buffer")
        flat = np.ctypeslib.as_array((ctypes.c_double * count).from_address(self.ptr))
        return flat.reshape(shape, order=order)

    def info(self):
        """(kind, huge_bytes): 1 for a huge-page mapping or 2 for cudaHostAlloc memory
        (huge pages unavailable), and the bytes now backed by huge pages (-1 unknown)."""
        kind, huge = ctypes.c_int(0), ctypes.c_longlong(0)
        rc = int(load().orth_gb300_host_buffer_info(self._p, ctypes.byref(kind), ctypes.byref(huge)))
        if rc != 0:
            raise RuntimeError(f"orth_gb300_host_buffer_info returned {rc}")
        return int(kind.value), int(huge.value)

    def close(self) -> None:
        if self._p.value:
            load().orth_gb300_host_free(self._p)
            self._p = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def last_host_timing() -> dict:
    """Timeline of this thread's last orth.h host-buffer run, in ms from its first
    device operation: X resident, compute done, Q back; and the call's wall time."""
    out = (ctypes.c_double * 4)()
    load().orth_gb300_last_host_timing(out)
    return {"x_resident_ms": out[0], "compute_done_ms": out[1], "q_back_ms": out[2], "wall_ms": out[3]}


def run_dev(variant: str, m: int, n: int, s: int, x_ptr: int, ldx: int, r_ptr: int, ldr: int,
            precision: int = FP64, stream: int = 0, want_status: bool = True):
    """Device-pointer entry point (orth_gb300_run_dev). Pointers are integers
    (e.g. ``tensor.data_ptr()``); ``stream`` is a cudaStream_t as an integer."""
    lib = load()
    st = Status()
    rc = lib.orth_gb300_run_dev(VARIANT_ID[variant], m, n, s, ctypes.c_void_p(x_ptr), ldx,
                                ctypes.c_void_p(r_ptr), ldr, precision, ctypes.c_void_p(stream),
                                ctypes.byref(st) if want_status else None)
    return int(rc), (st.as_dict() if want_status else None)


NOALLOC_TOO_LARGE = 5


def bcgsi2P1s_dev_noalloc(m: int, n: int, s: int, x_ptr: int, ldx: int, r_ptr: int, ldr: int,
                          stream: int = 0):
    """BCGSI+P-1S on device buffers with no device allocation (scratch lives in
    a fixed 16 MiB array inside the library). Returns (rc, status dict)."""
    st = Status()
    rc = load().orth_gb300_bcgsi2P1s_dev_noalloc(m, n, s, ctypes.c_void_p(x_ptr), ldx,
                                                 ctypes.c_void_p(r_ptr), ldr,
                                                 ctypes.c_void_p(stream), ctypes.byref(st))
    return int(rc), st.as_dict()


def set_host_precision(precision: int) -> int:
    """Precision of the orth.h entry points (FP64, SPLIT_BF16, SPLIT_BF16_FAST)."""
    return int(load().orth_gb300_set_host_precision(precision))


INTRA_TSQR = 0
INTRA_CHOLQR2 = 1


SHARD_ROWS = 8192


def shard_rows(m: int, size: int, rank: int):
    """This rank's (first row, row count) in a row-sharded run of m rows
    (orth_gb300_shard_rows; host arithmetic). Raises if a rank would get no rows."""
    r0, ms = ctypes.c_longlong(0), ctypes.c_longlong(0)
    rc = int(load().orth_gb300_shard_rows(m, size, rank, ctypes.byref(r0), ctypes.byref(ms)))
    if rc != 0:
        raise ValueError(f"no valid partition of {m} rows over {size} ranks")
    return r0.value, ms.value


def host_staged_allgather(gather_host):
    """An orth_gb300_allgather_fn that stages through host memory: it waits for the
    stream, copies `count` doubles of `send` to the host, calls
    gather_host(numpy array) -> list of every rank's arrays in rank order (for
    example torch.distributed.all_gather over gloo or MPI), and copies them back
    into `recv`. Keep the returned object alive while it is in use."""
    import torch

    def cb(ctx, send, recv, count, stream):
        try:
            n = int(count)
            st = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
            st.synchronize()
            host = np.empty(n, dtype=np.float64)
            cudart = _cudart()
            if cudart.cudaMemcpy(ctypes.c_void_p(host.ctypes.data), ctypes.c_void_p(send), n * 8, 2) != 0:
                return 1
            parts = gather_host(host)
            allh = np.ascontiguousarray(np.concatenate(parts))
            if cudart.cudaMemcpy(ctypes.c_void_p(recv), ctypes.c_void_p(allh.ctypes.data), allh.nbytes, 1) != 0:
                return 1
            return 0
        except Exception:
            return 1

    return ALLGATHER_FN(cb)


_cudart_lib = None


def _cudart():
    """The CUDA runtime this library links (for the host-staged exchange)."""
    global _cudart_lib
    if _cudart_lib is None:
        import glob
        import torch
        cands = sorted(glob.glob(os.path.join(os.path.dirname(torch.__file__), "lib", "libcudart.so*")))
        cands += sorted(glob.glob(os.path.join(os.path.dirname(os.path.dirname(torch.__file__)), "nvidia",
                                               "cuda_runtime", "lib", "libcudart.so*")))
        cands += ["libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"]
        for c in cands:
            try:
                _cudart_lib = ctypes.CDLL(c)
                break
            except OSError:
                continue
        if _cudart_lib is None:
            raise RuntimeError("libcudart not found")
        _cudart_lib.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        _cudart_lib.cudaMemcpy.restype = ctypes.c_int
    return _cudart_lib


def run_sharded(variant: str, m: int, n: int, s: int, x_ptr: int, ldx: int, r_ptr: int, ldr: int,
                rank: int, size: int, allgather, stream: int = 0):
    """One rank of a row-sharded run (orth_gb300_run_sharded): this rank's rows of
    X at x_ptr (device), a full R at r_ptr (device). Returns (rc, status dict)."""
    comm = Comm(rank, size, allgather, None)
    st = Status()
    rc = int(load().orth_gb300_run_sharded(VARIANT_ID[variant], m, n, s, ctypes.c_void_p(x_ptr), ldx,
                                           ctypes.c_void_p(r_ptr), ldr, ctypes.c_void_p(stream),
                                           ctypes.byref(comm), ctypes.byref(st)))
    return rc, st.as_dict()


def set_intra_ortho(mode: int) -> int:
    """IntraOrtho of the panels the reference factors with TSQR: INTRA_TSQR
    (default) or INTRA_CHOLQR2."""
    return int(load().orth_gb300_set_intra_ortho(mode))


def last_split_error() -> int:
    """Code of the last bounded wait of the split kernels that ran out (0 if none)."""
    return int(load().orth_gb300_last_split_error())


def split_supported(m: int, n: int, s: int) -> bool:
    return bool(load().orth_gb300_split_supported(m, n, s))


def gram_dev(m: int, na: int, b0: int, nb: int, x_ptr: int, ldx: int, c_ptr: int, ldc: int,
             precision: int = FP64, stream: int = 0) -> int:
    """C = X[:, 0:na]^T X[:, b0:b0+nb] on device buffers (one synchronization)."""
    return int(load().orth_gb300_gram_dev(m, na, b0, nb, ctypes.c_void_p(x_ptr), ldx,
                                          ctypes.c_void_p(c_ptr), ldc, precision,
                                          ctypes.c_void_p(stream)))


def accuracy_dev(m: int, n: int, x_ptr: int, ldx: int, q_ptr: int, ldq: int, r_ptr: int, ldr: int,
                 gram_precision: int = SPLIT_BF16, e_ptr: int = 0, lde: int = 0, stream: int = 0):
    """The reference's test_orth_accuracy (SRC/util.c:36-75) on device buffers.

    Returns (rc, loo_fro, residual_fro, x_fro): ||Q^T Q - I||_F, ||Q R - X||_F and
    ||X||_F. With e_ptr set, the symmetric n x n error Q^T Q - I is written there
    (ld lde) for a 2-norm.
    """
    out = (ctypes.c_double * 3)()
    rc = int(load().orth_gb300_accuracy_dev(m, n, ctypes.c_void_p(x_ptr), ldx, ctypes.c_void_p(q_ptr), ldq,
                                            ctypes.c_void_p(r_ptr), ldr, gram_precision,
                                            ctypes.c_void_p(e_ptr or None), lde or n, ctypes.c_void_p(stream),
                                            out))
    return rc, float(out[0]), float(out[1]), float(out[2])


def split_slice_dev(m: int, n: int, x_ptr: int, ldx: int, planes: int, digits_ptr: int, exp_ptr: int,
                    stream: int = 0) -> int:
    """The split form's BF16 digit planes of X (m x n, ld ldx) in the digit store's
    layout, and each column's scale exponent (orth_gb300_split_slice_dev)."""
    return int(load().orth_gb300_split_slice_dev(m, n, ctypes.c_void_p(x_ptr), ldx, planes,
                                                 ctypes.c_void_p(digits_ptr), ctypes.c_void_p(exp_ptr),
                                                 ctypes.c_void_p(stream)))


def poison_shared_memory(bits: int = 0x7FF8DEADBEEF0001, stream: int = 0) -> int:
    """Fill every SM's shared memory with a 64-bit pattern (default: a quiet NaN)."""
    return int(load().orth_gb300_poison_shared_memory(bits, ctypes.c_void_p(stream)))


def set_gram_chunk_rows(rows: int) -> None:
    """Rows per FP64 Gram chunk (0 restores the default chunking policy)."""
    load().orth_gb300_set_gram_chunk_rows(int(rows))


BATCH_TUNE = 1
BATCH_ONE_STREAM = 2
BATCH_STREAMS = 4


def _int_array(v):
    return (ctypes.c_int * len(v))(*[int(x) for x in v])


def batch_dry_run(ms, ns, ss) -> dict:
    """Stages, launches per run and device bytes of a batched plan (no GPU needed)."""
    st, la, wb = ctypes.c_longlong(0), ctypes.c_longlong(0), ctypes.c_longlong(0)
    rc = int(load().orth_gb300_batch_dry_run(len(ms), _int_array(ms), _int_array(ns), _int_array(ss),
                                             ctypes.byref(st), ctypes.byref(la), ctypes.byref(wb)))
    return {"rc": rc, "stages": st.value, "launches": la.value, "bytes": wb.value}


def split_batch_dry_run(ms, ns, ss, budget_bytes: int) -> dict:
    """Waves, launches per run and wave-buffer bytes of a staged split-precision
    batch (orth_gb300_split_batch_dry_run; no GPU needed)."""
    w, la, by = ctypes.c_int(0), ctypes.c_longlong(0), ctypes.c_longlong(0)
    rc = int(load().orth_gb300_split_batch_dry_run(len(ms), _int_array(ms), _int_array(ns), _int_array(ss),
                                                   int(budget_bytes), ctypes.byref(w), ctypes.byref(la),
                                                   ctypes.byref(by)))
    return {"rc": rc, "waves": w.value, "launches": la.value, "bytes": by.value}


def split_batch_plan(ms, ns, ss, free_bytes: int = -1, max_slots: int = 0) -> dict:
    """Slot count, slot of each matrix and enqueue order of a split-precision batch
    (orth_gb300_split_batch_plan; no GPU needed)."""
    c = len(ms)
    slot = (ctypes.c_int * c)()
    order = (ctypes.c_int * c)()
    S = int(load().orth_gb300_split_batch_plan(c, _int_array(ms), _int_array(ns), _int_array(ss), int(free_bytes),
                                            int(max_slots), slot, order))
    return {"slots": S, "slot_of": list(slot), "order": list(order)}


class Batch:
    """A batched BCGSI+P-1S plan over device buffers (orth_gb300_batch_*).

    x_ptrs[b]: device pointer of X_b (m x n column-major, ld ldx[b]); r_ptrs[b]:
    device pointer of R_b (n x n, ld ldr[b]). The plan captures the whole batch
    in one CUDA graph at creation; run() replays it.
    """

    def __init__(self, ms, ns, ss, x_ptrs, r_ptrs, ldx=None, ldr=None, precision=FP64, tune=True,
                 stream: int = 0, variant: str = "bcgsi2P1s", one_stream: bool = False, streams: bool = False):
        lib = load()
        self.count = len(ms)
        self._h = ctypes.c_void_p(0)
        xs = (ctypes.c_void_p * self.count)(*x_ptrs)
        rs = (ctypes.c_void_p * self.count)(*r_ptrs)
        lx = (ctypes.c_longlong * self.count)(*(ldx if ldx is not None else ms))
        lr = _int_array(ldr if ldr is not None else ns)
        self.rc = int(lib.orth_gb300_batch_create(ctypes.byref(self._h), VARIANT_ID[variant], self.count,
                                                  _int_array(ms), _int_array(ns), _int_array(ss), xs, lx, rs, lr,
                                                  precision, (BATCH_TUNE if tune else 0) | (BATCH_ONE_STREAM if one_stream else 0)
                                                  | (BATCH_STREAMS if streams else 0),
                                                  ctypes.c_void_p(stream)))

    def run(self, stream: int = 0) -> int:
        return int(load().orth_gb300_batch_run(self._h, ctypes.c_void_p(stream)))

    def status(self):
        steps, infos, nb = (ctypes.c_int * self.count)(), (ctypes.c_int * self.count)(), ctypes.c_int(0)
        rc = int(load().orth_gb300_batch_status(self._h, steps, infos, ctypes.byref(nb)))
        return rc, list(steps), list(infos), nb.value

    def info(self) -> dict:
        la, wb, gn = ctypes.c_longlong(0), ctypes.c_longlong(0), ctypes.c_int(0)
        tuned = (ctypes.c_int * 6)()
        load().orth_gb300_batch_info(self._h, ctypes.byref(la), ctypes.byref(wb), ctypes.byref(gn), tuned)
        return {"launches": la.value, "bytes": wb.value, "graph_nodes": gn.value,
                "tuned": {4: (tuned[0], tuned[1]), 8: (tuned[2], tuned[3]), 16: (tuned[4], tuned[5])}}

    def close(self) -> None:
        if self._h:
            load().orth_gb300_batch_destroy(self._h)
            self._h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sync_count(variant: str, n: int, s: int) -> int:
    return int(load().orth_gb300_sync_count(VARIANT_ID[variant], n, s))


def last_launch_count() -> int:
    return int(load().orth_gb300_last_launch_count())


def last_reduction_count() -> int:
    """Device-wide reductions (synchronizations) the last run on this thread launched."""
    return int(load().orth_gb300_last_reduction_count())


PROFILE_CLASSES = ("gram", "update", "small", "tsqr", "slice")


def profile(on: bool) -> None:
    """Enable (and reset) or disable per-kernel-class event timing."""
    load().orth_gb300_profile(1 if on else 0)


def profile_read() -> dict:
    """Per class since profile(True): ms, launches, algorithmic flops and bytes
    (FP64-equivalent), and the bytes the kernels as built move (digit planes for
    the split forms)."""
    k = len(PROFILE_CLASSES)
    ms = (ctypes.c_double * k)()
    ln = (ctypes.c_longlong * k)()
    fl = (ctypes.c_double * k)()
    by = (ctypes.c_double * k)()
    rc = load().orth_gb300_profile_read(ms, ln, fl, by)
    if rc != 0:
        raise RuntimeError(f"orth_gb300_profile_read failed: {rc}")
    tr = (ctypes.c_double * k)()
    calls = (ctypes.c_longlong * k)()
    load().orth_gb300_profile_traffic(tr, calls)
    return {c: {"ms": ms[i], "launches": ln[i], "flops": fl[i], "bytes": by[i], "traffic": tr[i],
                "calls": calls[i]}
            for i, c in enumerate(PROFILE_CLASSES)}


def fp64_peak_tflops() -> float:
    """FP64 pipe throughput of the current GPU, measured by a DFMA loop."""
    v = ctypes.c_double(0.0)
    rc = load().orth_gb300_fp64_peak_probe(ctypes.byref(v))
    if rc != 0:
        raise RuntimeError(f"fp64 probe failed: {rc}")
    return float(v.value)


def reserve(m: int, n: int, s: int) -> int:
    return int(load().orth_gb300_reserve(m, n, s))


def release() -> None:
    load().orth_gb300_release()


def version() -> str:
    return load().orth_gb300_version().decode()
