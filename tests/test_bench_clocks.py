"""bench.py's clock record: parsing of the nvidia-smi samples and the
throttle reasons a run is judged by (CPU only, no GPU or nvidia-smi needed)."""
import time

import bench


def _sampler(lines):
    c = bench.ClockSampler(0)
    c.lines = list(lines)
    return c


def test_summary_median_max_and_reasons():
    lines = [
        "0, 2070, 2070, 910.2, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1290.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1300.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
    ]
    s = _sampler(lines).summary()
    assert s["samples"] == 3
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]


def test_summary_reports_thermal_and_hw_slowdown():
    lines = ["0, 1500, 2070, 1400, 0x48, Active, Not Active, Active, Not Active"]
    s = _sampler(lines).summary()
    assert s["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    assert s["sm_mhz"] == 1500.0


def test_summary_skips_malformed_lines_and_handles_none():
    s = _sampler(["", "0, [N/A], 2070, 1, 0x0, a, b, c, d", "garbage"]).summary()
    assert s == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_sampler_without_a_gpu_returns_promptly():
    """Entering the sampler waits at most a few seconds for a first sample;
    with no GPU (or no nvidia-smi) it records nothing and does not fail."""
    t0 = time.time()
    c = bench.ClockSampler(0).__enter__()
    c.__exit__(None, None, None)
    assert time.time() - t0 < 10.0
    assert c.summary()["samples"] >= 0
