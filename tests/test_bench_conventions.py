"""The bench line's fixed conventions, on the CPU: the whole-step roofline's
algorithmic bytes per phase (sort 28 B/particle + 8 B per cell, deposit 12
B/particle + 4 B per mesh point, two transforms of two passes each reading and
writing the half spectrum, interpolation 24 B/particle + three force grids),
20 FP32 flops per in-range pair, and the HBM peak taken from the measured
peaks file when present."""
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
