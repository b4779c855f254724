"""The structured per-step log: JSON lines a box run and a serving loop write
(one record per step; one per tick and per finished job)."""
import io

import numpy as np
import pytest

from cuco_gb300 import steplog


def test_records_are_json_lines(tmp_path):
    path = str(tmp_path / "log.jsonl")
    log = steplog.StepLog(path)
    log.write("box_step", step=0, a=0.02, phase_ms={"total": 1.5}, particle_updates_per_s=1e9)
    log.write("tick", tick=1, running=3, queued=0, updates=12)
    log.close()
    recs = steplog.read(path)
    assert [r["kind"] for r in recs] == ["box_step", "tick"]
    assert recs[0]["phase_ms"]["total"] == 1.5 and recs[1]["running"] == 3
    buf = io.StringIO()
    steplog.StepLog(buf).write("job_done", job=4, latency=2.5)
    assert '"job": 4' in buf.getvalue() and buf.getvalue().endswith("\n")


@pytest.mark.gpu
def test_box_run_logs_every_step(tmp_path):
    from cuco_gb300 import Box, BoxConfig, fixed_step_schedule, ics
    ic = ics.zeldovich(16, 50.0, 49.0, 3)
    box = Box(BoxConfig(n=ic.n, pm_grid=32, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                        softening=2.8 * 0.03 * ic.boxsize / 16))
    box.set_state(ic.pos, ic.canonical_velocity())
    a, drift, kick = fixed_step_schedule(ic.a, 1.0, 5)
    path = str(tmp_path / "steps.jsonl")
    log = steplog.StepLog(path)
    box.run(drift, kick, a=a, log=log)
    log.close()
    recs = steplog.read(path)
    assert [r["step"] for r in recs] == list(range(6))
    assert np.allclose([r["a"] for r in recs], a)
    for r in recs:
        assert r["phase_ms"]["total"] > 0 and r["particle_updates_per_s"] > 0
        assert set(r["phase_ms"]) == set(Box.PHASES)
    box.close()
