"""Total force (short range + PM) of the engine against the FP64 Ewald oracle,
beside the reference method's own error against it (its force path restated
by the oracle, bit-exact with the reference's CPU code: the method floor).

Small box (32^3 particles, L = 100 Mpc/h, M = 64, softening 0.03 of the mean
spacing): every particle is a target, at the initial conditions (z = 49),
after 10 steps, and at z = 0 after a 200-step run.  The mid-size box
(128^3, M = 256) is covered in test_gpu_precision_form.py on a 4096-particle
subsample.

Error metric: rms relative sqrt(sum |a - a_ewald|^2 / sum |a_ewald|^2) over the
targets, printed with the median and 99th percentile of the per-particle
relative error |a_i - a_ewald,i| / |a_ewald,i|.  Bars (on the rms): the plain form is the reference's method computed to 1e-4 of
the reference's own force, so its error must equal the floor within 2e-4; the
precision form (within 1e-3 of the reference's force) within 1.5e-3 of it;
and wherever the floor is below 8e-4 both must be at most 1e-3."""
import numpy as np
import pytest

import oracle
from cuco_gb300 import Box, BoxConfig, fixed_step_schedule, ics
from cuco_gb300.engine import MODE_FIXED
from conftest import err_stats
from helpers import softening_h

pytestmark = pytest.mark.gpu

NS, BOX_MPC, M, Z0, SEED = 32, 100.0, 64, 49.0, 1


def ewald_table(port, pos, ic, soft, M, targets, nthreads=16):
    """{floor, plain, precision}: total-force errors against Ewald (err_stats)."""
    L = float(np.float32(ic.boxsize))
    mass = float(np.float32(ic.mass))
    ew = port.ewald(pos.astype(np.float64), mass, ics.G_INTERNAL, L, soft, pos[targets].astype(np.float64),
                    nthreads)
    p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, M, soft)
    ref = port.pp_targets(pos, targets, p, M, nthreads).astype(np.float64) + \
        port.pm(pos, p, M, nthreads)[targets].astype(np.float64)
    out = {"floor": err_stats(ref, ew)}
    for mode, name in ((0, "plain"), (MODE_FIXED, "precision")):
        box = Box(BoxConfig(n=ic.n, pm_grid=M, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                            softening=soft, mode=mode))
        box.set_state(pos)
        box.forces()
        _, _, app, apm = box.get_state()
        box.close()
        out[name] = err_stats(app[targets].astype(np.float64) + apm[targets], ew)
    return out


def check_against_floor(t):
    r = {k: v["rms"] for k, v in t.items()}
    assert abs(r["plain"] - r["floor"]) < 2e-4, t
    assert r["precision"] < r["floor"] + 1.5e-3, t
    if r["floor"] < 8e-4:
        assert r["plain"] <= 1e-3 and r["precision"] <= 1e-3, t


def table_line(label, t):
    """One line: rms / median / p99 of the floor and of both forms."""
    return label + ": " + "  ".join(f"{k} {v['rms']:.3e}/{v['median']:.3e}/{v['p99']:.3e}" for k, v in t.items()) \
        + "  (rms/median/p99)"


@pytest.fixture(scope="module")
def small_states():
    ic = ics.zeldovich(NS, BOX_MPC, Z0, SEED)
    soft = softening_h(ic.boxsize, NS)
    box = Box(BoxConfig(n=ic.n, pm_grid=M, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                        softening=soft))
    box.set_state(ic.pos, ic.canonical_velocity())
    states = {"z49": ic.pos.copy()}
    _, drift, kick = fixed_step_schedule(ic.a, 1.0, 200)
    for s in range(201):
        box.step(drift[s], kick[s])
        if s == 10:
            states["step10"] = box.get_state()[0]
    states["z0"] = box.get_state()[0]
    box.close()
    return ic, soft, states


@pytest.mark.parametrize("state", ["z49", "step10", "z0"])
def test_small_box_vs_ewald(port, small_states, state):
    ic, soft, states = small_states
    pos = states[state]
    t = ewald_table(port, pos, ic, soft, M, np.arange(ic.n))
    print(table_line(f"EWALD 32^3 M=64 {state}", t))
    check_against_floor(t)
