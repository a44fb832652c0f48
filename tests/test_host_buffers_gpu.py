"""GPU tests of the library's huge-page host buffers (orth_gb300_host_alloc).

The orth.h entry points take X and R in any host memory; the buffers from
orth_gb300_host_alloc are page-locked and backed by huge pages, so the copies
run at the host link's full rate. Checked through the C ABI:
  * a fresh buffer reads as zero, is page-locked (the CUDA driver reports it as
    host memory it knows), and is released once (a second free returns 2);
  * a large buffer is on huge pages, or comes from cudaHostAlloc where the host
    cannot give them;
  * an orth.h call on such buffers gives Q and R bit-identical to the same call
    on ordinary (pageable) numpy buffers, in FP64 and in the 56-bit split form:
    only the copies differ, not the device computation.
"""
import ctypes

import numpy as np
import pytest

from bcgs_gb300 import inputs, orth

pytestmark = pytest.mark.gpu


def test_host_buffer_is_zeroed_pinned_and_freed_once(lib):
    torch = pytest.importorskip("torch")
    torch.cuda.init()
    hb = orth.HostBuffer((3 << 20) + 24)
    a = hb.array((3 << 17,))
    assert a.shape == (3 << 17,) and not a.any()
    a[:] = np.arange(a.size, dtype=np.float64)
    # The driver knows the range as host memory (cudaPointerGetAttributes type 1).
    cudart = orth._cudart()
    attr = (ctypes.c_int * 32)()       # struct cudaPointerAttributes is 88 bytes; type first
    cudart.cudaPointerGetAttributes.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    cudart.cudaPointerGetAttributes.restype = ctypes.c_int
    assert cudart.cudaPointerGetAttributes(ctypes.addressof(attr), ctypes.c_void_p(hb.ptr)) == 0
    assert attr[0] == 1, list(attr)[:4]
    # Round trip through the device with a copy engine.
    d = torch.empty(a.size, dtype=torch.float64, device="cuda")
    d.copy_(torch.from_numpy(a))
    back = d.cpu().numpy()
    assert np.array_equal(back, a)
    kind, huge = hb.info()
    assert kind in (1, 2) and (huge >= 0 or huge == -1)
    p = hb.ptr
    hb.close()
    assert lib.orth_gb300_host_free(ctypes.c_void_p(p)) == 2


def test_large_host_buffer_is_huge_page_backed_or_cuda_host_alloc(lib):
    """A buffer of 1 GiB is either a mapping mostly on huge pages or, where the host
    cannot give them, cudaHostAlloc memory; it reads as zero either way."""
    torch = pytest.importorskip("torch")
    torch.cuda.init()
    hb = orth.HostBuffer(1 << 30)
    try:
        kind, huge = hb.info()
        if kind == 1 and huge >= 0:
            assert huge >= 3 * (1 << 30) // 4
        else:
            assert kind == 2 or huge == -1
        a = hb.array((1 << 27,))
        assert not a[:: 4096].any() and not a[-1]
    finally:
        hb.close()


@pytest.mark.parametrize("precision", ["fp64", "split7"])
def test_orth_h_on_host_buffers_matches_pageable(lib, precision):
    m, n, s = 300001, 96, 16
    X = inputs.graded_host(m, n, 1e6, seed=21)
    prec = orth.FP64 if precision == "fp64" else orth.SPLIT_BF16
    orth.set_host_precision(prec)
    try:
        Xp = np.asfortranarray(X.copy())
        Rp = np.zeros((n, n), order="F")
        assert orth.call("bcgsi2P1s", m, n, s, Xp, m, Rp, n) == 0
        hx, hr = orth.HostBuffer(m * n * 8), orth.HostBuffer(n * n * 8)
        Xh, Rh = hx.array((m, n)), hr.array((n, n))
        Xh[:] = X
        assert orth.call("bcgsi2P1s", m, n, s, Xh, m, Rh, n) == 0
        assert np.array_equal(Xh, Xp)
        assert np.array_equal(Rh, Rp)
        t = orth.last_host_timing()
        assert 0 < t["x_resident_ms"] <= t["wall_ms"] and t["q_back_ms"] <= t["wall_ms"] + 1.0
        hx.close()
        hr.close()
    finally:
        orth.set_host_precision(orth.FP64)
