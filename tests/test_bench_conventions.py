"""The bench line's fixed conventions, on the CPU: the whole-step roofline's
algorithmic bytes per phase (sort 28 B/particle + 8 B per cell, deposit 12
B/particle + 4 B per mesh point, two transforms of two passes each reading and
writing the half spectrum, interpolation 24 B/particle + three force grids),
20 FP32 flops per in-range pair, and the HBM peak taken from the measured
peaks file when present; the clocks record summarised from nvidia-smi
samples; and the reference arm's JSON line, which runs on the CPU."""
import json
import os

import pytest

import bench


def test_step_roofline_bytes_and_fraction():
    n, M, G, pairs, ms, tf = 2097152, 256, 64, 1.776e8, 1.64, 76.2
    r = bench.step_roofline(n, M, G, pairs, ms, tf)
    b = r["algorithmic_bytes"]
    assert b["sort"] == 28 * n + 8 * G ** 3
    assert b["deposit"] == 12 * n + 4 * M ** 3
    assert b["fft"] == 2 * 2 * 2 * 8 * M * M * (M // 2 + 1)
    assert b["interpolation"] == 24 * n + 12 * M ** 3
    hbm = r["hbm_peak_gbs"]
    ideal = {k: 1e3 * v / (hbm * 1e9) for k, v in b.items()}
    ideal["pair_force"] = 1e3 * 20.0 * pairs / (tf * 1e12)
    assert r["ideal_ms"] == pytest.approx(sum(ideal.values()), rel=1e-4)
    assert r["frac"] == pytest.approx(sum(ideal.values()) / ms, rel=1e-4)
    assert 0.0 < r["frac"] < 1.0


def test_hbm_peak_source():
    hbm, kind = bench.measured_hbm_gbs()
    path = os.path.join(os.path.dirname(os.path.abspath(bench.__file__)), "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            assert kind == "measured" and hbm == float(json.load(f)["hbm_gbs"])
    else:
        assert kind == "fallback" and hbm == 6800.0


def test_reference_arm_line():
    """`bench.py --impl reference` (the CPU force path, no GPU) prints one JSON
    line with the GPU arm's metric and unit, `impl`, a cpu_baseline describing
    the run and an e2e of zero copied bytes; warm-up is held at 3 or more."""
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(bench.__file__))
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=here, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "particle-updates/s" and d["unit"] == "particle-updates/s"
    assert d["steps"] == 1 and d["warmup"] >= 3 and d["higher_is_better"] is True
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"]


def test_clock_summary():
    """The clocks record of the bench line from nvidia-smi samples: the median
    SM clock under load, the maximum, and every throttle reason seen active
    (unparseable readings skipped)."""
    cs = bench.ClockSampler()
    na, act = "Not Active", "Active"
    cs.samples = [["2070", "2070", "901.2", na, na, na, na],
                  ["1980", "2070", "1398.0", na, na, na, act],
                  ["[N/A]", "2070", "1400.0", na, na, na, act],
                  ["2055", "[N/A]", "1200.0", na, act, na, na]]
    s = cs.stop()
    assert s["sm_mhz"] == 2055.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 4
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert bench.ClockSampler().stop()["reasons"] == ["unsampled"]
