"""CPU tests of bench.py's host-side logic: the clock record that decides whether
a run is kept (median SM clock under load, throttle reasons seen), and the
algorithmic byte and flop counts behind `hbm_gbs_alg` and `tflops_alg`."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    # Imported inside the tests: bench.py sets CUDA_DEVICE_MAX_CONNECTIONS on
    # import, which must not leak into the GPU tests collected in the same run.
    sys.path.insert(0, ROOT)
    import bench
    return bench


def _sampler(lines):
    c = _bench().ClockSampler(0)
    c.lines = list(lines)
    return c


def test_clock_summary_median_and_reasons():
    # index, clocks.sm, clocks.max.sm, power.draw, active mask, hw_slowdown,
    # hw_thermal_slowdown, sw_thermal_slowdown, sw_power_cap
    lines = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1390.2, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    s = _sampler(lines).summary()
    assert s["samples"] == 3
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_summary_flags_thermal_and_empty():
    s = _sampler(["0, 1500, 2070, 1000, 0x40, Not Active, Active, Not Active, Not Active"]).summary()
    assert s["reasons"] == ["hw_thermal_slowdown"] and s["sm_mhz"] == 1500.0
    e = _sampler([]).summary()
    assert e["samples"] == 0 and e["sm_mhz"] is None and e["reasons"] == []


def test_algorithmic_counts_at_config1():
    bench = _bench()
    m, n, s = 1 << 23, 512, 16
    # One read of Q_{1:k-1} per block step plus reading X, writing Q and writing
    # and reading U once: 8 m (s P (P-1)/2 + 4 n) with P = n / s.
    assert bench.alg_bytes_p1s(m, n, s) == 8.0 * m * (16 * 32 * 31 / 2 + 4 * 512)
    assert abs(bench.alg_bytes_p1s(m, n, s) - 6.70e11) / 6.70e11 < 0.01
    assert bench.alg_flops_p1s(m, n, s) == 4.0 * m * n * n + 8.0 * m * n * s
    assert abs(bench.alg_flops_p1s(m, n, s) - 9.35e12) / 9.35e12 < 0.01


def test_reference_arm_runs_full_size_steps_within_budget():
    """--impl reference times whole QRs of the configured size (no scaling), runs
    no more steps than asked or than the budget allows, says how many ran, and
    runs the warm-up steps asked for."""
    import json
    import subprocess
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--m", "8192",
                        "--n", "64", "--s", "16", "--steps", "3", "--warmup", "2", "--ref-budget-s", "60"],
                       capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "ms"
    assert 1 <= line["steps"] <= 3 and line["steps_requested"] == 3 and line["warmup"] == 2
    assert len(line["step_ms"]) == line["steps"]
    assert abs(sum(line["step_ms"]) / line["steps"] - line["value"]) < 0.2
    assert "m=8192" in line["config"]["workload"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
