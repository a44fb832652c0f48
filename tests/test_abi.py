"""CPU tests of the C-ABI library: it builds, loads, exports every declared
entry point, and applies the reference's argument checks before touching a GPU."""
import os
import re
import subprocess

import numpy as np

from bcgs_gb300 import orth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("orth.h", "orth_gb300.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|void|long long|const char\s*\*)\s*\**\s*(\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", orth.lib_path()], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    declared = declared_functions()
    assert {"bcgsi2P1s", "bcgsi21s", "bcgspipi2", "bcgsi2", "bcgsi2P2s"} <= declared
    missing = declared - exported
    assert not missing, missing


def test_lwork_too_small_returns_1(lib, capfd):
    m, n, s = 64, 16, 4
    X = np.zeros((m, n), order="F")
    R = np.zeros((n, n), order="F")
    for v in orth.VARIANTS:
        need = orth.lwork_min(m, n, s, v)
        rc = orth.call(v, m, n, s, X, m, R, n, lwork=need - 1)
        assert rc == 1
    assert "Work space is too small" in capfd.readouterr().out


def test_invalid_arguments_return_2(lib):
    X = np.zeros((64, 16), order="F")
    R = np.zeros((16, 16), order="F")
    assert orth.call("bcgsi2P1s", 64, 16, 9, X, 64, R, 16) == 2      # n < 2s
    assert orth.call("bcgsi2P1s", 64, 16, 4, X, 63, R, 16) == 2      # ld < m
    assert orth.call("bcgsi2P1s", 64, 16, 4, X, 64, R, 15) == 2      # ldR < n
    assert orth.call("bcgsi2P1s", 64, 16, 0, X, 64, R, 16) == 2      # s < 1


def test_sync_counts(lib):
    # BCGSI+P-1S / BCGSI+A-1S / BCGSI+P-2S: two synchronizations in the first
    # step, then exactly one per block step; PIPI and BCGSI+ two per step.
    n, s = 512, 16
    p = (n - s + s - 1) // s
    assert orth.sync_count("bcgsi2P1s", n, s) == p + 1
    assert orth.sync_count("bcgsi21s", n, s) == p + 1
    assert orth.sync_count("bcgsi2P2s", n, s) == p + 1
    assert orth.sync_count("bcgspipi2", n, s) == 2 * p
    assert orth.sync_count("bcgsi2", n, s) == 2 * p


def test_version(lib):
    assert "sm_103a" in orth.version()


def test_host_timing_is_zero_before_any_host_run(lib):
    # The timeline is per thread and set only by a successful host-buffer run; a
    # fresh thread reads zeros without touching the GPU.
    import threading
    got = {}
    t = threading.Thread(target=lambda: got.update(orth.last_host_timing()))
    t.start()
    t.join()
    assert got == {"x_resident_ms": 0.0, "compute_done_ms": 0.0, "q_back_ms": 0.0, "wall_ms": 0.0}


def test_split_shape_support(lib):
    # Split precision takes s <= 64 with n >= 2s and at least one 128-row tile.
    assert orth.split_supported(1 << 20, 512, 16)
    assert orth.split_supported(1 << 20, 512, 64)
    assert not orth.split_supported(1 << 20, 512, 65)
    assert not orth.split_supported(1 << 20, 100, 64)
    assert not orth.split_supported(127, 32, 4)


def test_timeout_probe_rejects_code_zero(lib):
    # Code 0 means "no error" and is rejected before any CUDA call.
    assert orth.timeout_probe(0)[0] == 2


def test_host_buffer_argument_checks(lib):
    """orth_gb300_host_alloc / _free reject bad arguments before any CUDA call."""
    import ctypes
    p = ctypes.c_void_p(0)
    assert lib.orth_gb300_host_alloc(ctypes.c_size_t(0), ctypes.byref(p)) == 2 and not p.value
    assert lib.orth_gb300_host_alloc(ctypes.c_size_t(64), None) == 2
    assert lib.orth_gb300_host_free(None) == 0
    assert lib.orth_gb300_host_free(ctypes.c_void_p(0x12345000)) == 2   # not from orth_gb300_host_alloc
    kind, huge = ctypes.c_int(0), ctypes.c_longlong(0)
    assert lib.orth_gb300_host_buffer_info(None, ctypes.byref(kind), ctypes.byref(huge)) == 2
    assert lib.orth_gb300_host_buffer_info(ctypes.c_void_p(0x12345000), ctypes.byref(kind), ctypes.byref(huge)) == 2


def test_split_slice_argument_checks(lib):
    """orth_gb300_split_slice_dev rejects bad arguments before any CUDA call."""
    assert orth.split_slice_dev(0, 4, 0, 1, 7, 0, 0) == 2          # m < 1
    assert orth.split_slice_dev(16, 4, 0, 16, 7, 0, 0) == 2         # null buffers
    assert orth.split_slice_dev(16, 4, 0x1000, 8, 7, 0x1000, 0x1000) == 2   # ldX < m
    assert orth.split_slice_dev(16, 4, 0x1000, 16, 5, 0x1000, 0x1000) == 2  # planes not 6 or 7
