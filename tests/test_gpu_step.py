"""A full step (drift, wrap, keys, sort, PM, short range, kick) against the
oracle, and the device arithmetic of drift/kick against its host restatement."""
import numpy as np
import pytest

import oracle
from cuco_gb300 import Box, BoxConfig, fixed_step_schedule, ics
from helpers import softening_h, zeldovich
from conftest import rms_rel

pytestmark = pytest.mark.gpu


def oracle_step(port, pos, vel, p, M, G, drift, kick):
    """predict.c + accel.c + timestep.c for one global step, on the CPU."""
    L = np.float64(np.float32(p.boxsize))
    x = (pos.astype(np.float64) + vel.astype(np.float64) * drift).astype(np.float32)
    x = np.where(x < 0, (x.astype(np.float64) + L).astype(np.float32), x)
    x = np.where(x >= np.float32(L), (x.astype(np.float64) - L).astype(np.float32), x)
    app = port.pp(x, p, G, 8)
    apm = port.pm(x, p, M, 8)
    dv = (app.astype(np.float64) * kick).astype(np.float32)
    v = (vel + dv).astype(np.float32)
    v = (v.astype(np.float64) + apm.astype(np.float64) * kick).astype(np.float32)
    return x, v, app, apm


def test_steps_match_oracle(port):
    ic = zeldovich(32, 100.0, seed=11)
    M, G = 64, 64
    soft = softening_h(ic.boxsize, 32)
    box = Box(BoxConfig(n=ic.n, pm_grid=M, cell_grid=G, boxsize=ic.boxsize, mass=ic.mass,
                        G=ics.G_INTERNAL, softening=soft))
    vel0 = ic.canonical_velocity()
    box.set_state(ic.pos, vel0)
    a, drift, kick = fixed_step_schedule(ic.a, 0.1, 10)
    p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, M, soft)
    x, v = ic.pos.copy(), vel0.copy()
    for s in range(4):
        box.step(drift[s], kick[s], kick[s])
        x, v, app, apm = oracle_step(port, x, v, p, M, G, drift[s], kick[s])
        gx, gv, gpp, gpm = box.get_state()
        assert rms_rel(gpp, app) < 1e-4
        assert rms_rel(gpm, apm) < 1e-4
        assert rms_rel(gv, v) < 1e-4
        # positions agree to float rounding of the drift
        d = np.abs(gx - x)
        d = np.minimum(d, ic.boxsize - d)
        assert d.max() < 1e-3 * ic.boxsize / 32
    box.close()


def test_fixed_schedule_closes_leapfrog():
    a, drift, kick = fixed_step_schedule(0.02, 1.0, 200)
    from cuco_gb300 import cosmo_factors
    d_tot, k_tot = cosmo_factors(0.02, 1.0)
    assert drift.sum() == pytest.approx(d_tot, rel=1e-10)
    assert kick.sum() == pytest.approx(k_tot, rel=1e-10)
    assert a[-1] == pytest.approx(1.0)


@pytest.mark.parametrize("mode", [0, 1])
def test_split_and_joined_schedules_agree(monkeypatch, mode):
    """A box runs its short range either beside the PM's tail (split launch,
    the PM half of the kick after both) or after the PM (both halves of the
    kick in the short range's epilogue), by particle count; the two schedules
    give the same state bit for bit, through steps with kicks and through a
    plain force pass."""
    from cuco_gb300.engine import MODE_FIXED
    ic = zeldovich(48, 150.0, seed=12)
    M, G = 96, 48
    soft = softening_h(ic.boxsize, 48)
    vel0 = ic.canonical_velocity()
    a, drift, kick = fixed_step_schedule(ic.a, 0.2, 6)
    out = []
    for threshold in ("0", str(1 << 30)):  # always split, never split
        monkeypatch.setenv("CUCO_SPLIT_MIN_PARTICLES", threshold)
        box = Box(BoxConfig(n=ic.n, pm_grid=M, cell_grid=G, boxsize=ic.boxsize, mass=ic.mass,
                            G=ics.G_INTERNAL, softening=soft, mode=MODE_FIXED if mode else 0))
        box.set_state(ic.pos, vel0)
        for s in range(5):
            box.step(drift[s], kick[s], kick[s])
        stepped = box.get_state()
        box.forces()
        out.append((stepped, box.get_state()))
        box.close()
    for x, y in zip(out[0][0] + out[0][1], out[1][0] + out[1][1]):
        assert np.array_equal(x, y)
