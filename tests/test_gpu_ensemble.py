"""The batched form (cuco_ensemble_*): many boxes in one launch per phase.

Each box of an ensemble must get exactly the forces it gets alone: the short
range runs the same per-segment code on the same cell-ordered sources, and
the PM deposit adds integer weights (order-independent), so both are compared
bit for bit with a single box of the same cell grid.  Meshes that are not
powers of two (2 x the particle grid, as the batched workload has them) are
checked against the oracle, whose FFT falls back to the DFT by definition for
them.  Steps replayed from the captured graph must equal single boxes stepped
alone, bit for bit.
"""
import numpy as np
import pytest

import oracle
from cuco_gb300 import Box, BoxConfig, fixed_step_schedule, ics
from cuco_gb300.engine import MODE_FIXED, MODE_PLAIN
from cuco_gb300.ensemble import Ensemble
from conftest import rms_rel

pytestmark = pytest.mark.gpu

SPECS = [(16, 32, 60.0, 1), (20, 40, 120.0, 2), (24, 48, 200.0, 3), (18, 36, 90.0, 4)]


def soft(L, n_side):
    return float(np.float32(2.8 * np.float32(0.025 * L * 1000.0 / n_side)))


def make(specs, mode, cell_grid=None):
    ics_, cfgs = [], []
    for n_side, M, L, seed in specs:
        ic = ics.zeldovich(n_side, L, 49.0, seed)
        ics_.append(ic)
        cfgs.append(BoxConfig(n=ic.n, pm_grid=M, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                              softening=soft(L, n_side), mode=mode, cell_grid=cell_grid))
    return ics_, cfgs


def test_ensemble_forces_match_single_boxes():
    ics_, cfgs = make(SPECS, MODE_FIXED)
    ens = Ensemble(cfgs)
    for b, ic in enumerate(ics_):
        ens.set_state(b, ic.pos)
    ens.forces()
    for b, (ic, c) in enumerate(zip(ics_, cfgs)):
        G, P, B = ens.plan(b)
        assert G >= 8 and P >= 1 and B >= 1
        _, _, app, apm = ens.get_state(b)
        c1 = BoxConfig(**{**c.__dict__, "cell_grid": G})
        box = Box(c1)
        box.set_state(ic.pos)
        box.forces()
        _, _, app1, apm1 = box.get_state()
        box.close()
        assert np.array_equal(app, app1), f"box {b}: short range differs from the box alone"
        assert np.array_equal(apm, apm1), f"box {b}: PM differs from the box alone"
    ens.close()


def test_ensemble_mixed_radix_meshes_vs_oracle(port):
    specs = [(24, 48, 100.0, 5), (30, 60, 150.0, 6), (20, 40, 80.0, 7)]
    ics_, cfgs = make(specs, 0)
    ens = Ensemble(cfgs)
    for b, ic in enumerate(ics_):
        ens.set_state(b, ic.pos)
    ens.forces()
    for b, (ic, c) in enumerate(zip(ics_, cfgs)):
        _, _, app, apm = ens.get_state(b)
        p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, c.pm_grid, c.softening)
        e_pp = rms_rel(app, port.pp(ic.pos, p, c.pm_grid // 2, 8))
        e_pm = rms_rel(apm, port.pm(ic.pos, p, c.pm_grid, 8))
        print(f"M={c.pm_grid}: pp {e_pp:.2e} pm {e_pm:.2e}")
        assert e_pp < 1e-4 and e_pm < 1e-4
    ens.close()


def test_single_box_mixed_radix_pm_vs_oracle(port):
    ic = ics.zeldovich(30, 100.0, 49.0, 9)
    for M in (60, 90):
        box = Box(BoxConfig(n=ic.n, pm_grid=M, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                            softening=soft(100.0, 30), cell_grid=M // 4))
        box.set_state(ic.pos)
        box.forces(pm=True, pp=False)
        apm = box.get_state()[3]
        box.close()
        p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, M, soft(100.0, 30))
        assert rms_rel(apm, port.pm(ic.pos, p, M, 8)) < 1e-4


@pytest.mark.parametrize("M", [64, 256, 512])
def test_single_box_register_fft_pm_vs_oracle(port, M):
    """Power-of-two meshes take the register transforms (16- and 32-point
    DFTs at M = 512)."""
    ic = ics.zeldovich(24, 80.0, 49.0, 10)
    box = Box(BoxConfig(n=ic.n, pm_grid=M, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                        softening=soft(80.0, 24), cell_grid=max(8, M // 8)))
    box.set_state(ic.pos)
    box.forces(pm=True, pp=False)
    apm = box.get_state()[3]
    box.close()
    p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, M, soft(80.0, 24))
    e = rms_rel(apm, port.pm(ic.pos, p, M, 16))
    print(f"M={M}: pm {e:.2e}")
    assert e < 1e-4


def test_ensemble_large_mesh_matches_single_box():
    """A 512 mesh runs in the ensemble's own large-transform kernels; the box
    still gets exactly what it gets alone."""
    ics_, cfgs = make([(24, 512, 80.0, 11), (16, 32, 60.0, 1)], MODE_FIXED)
    ens = Ensemble(cfgs)
    for b, ic in enumerate(ics_):
        ens.set_state(b, ic.pos)
    ens.forces()
    for b, (ic, c) in enumerate(zip(ics_, cfgs)):
        _, _, _, apm = ens.get_state(b)
        box = Box(BoxConfig(**{**c.__dict__, "cell_grid": ens.plan(b)[0]}))
        box.set_state(ic.pos)
        box.forces()
        apm1 = box.get_state()[3]
        box.close()
        assert np.array_equal(apm, apm1), f"box {b}: PM differs from the box alone"
    ens.close()


def test_ensemble_graph_steps_track_single_boxes():
    ics_, cfgs = make(SPECS, MODE_FIXED)
    ens = Ensemble(cfgs)
    for b, ic in enumerate(ics_):
        ens.set_state(b, ic.pos, ic.canonical_velocity())
    a, drift, kick = fixed_step_schedule(ics_[0].a, 0.05, 4)
    for s in range(5):  # the first call captures the graph, the rest replay it
        ens.step(drift[s], kick[s])
    ens.sync()
    for b, (ic, c) in enumerate(zip(ics_, cfgs)):
        pos, vel, _, _ = ens.get_state(b)
        box = Box(BoxConfig(**{**c.__dict__, "cell_grid": ens.plan(b)[0]}))
        box.set_state(ic.pos, ic.canonical_velocity())
        for s in range(5):
            box.step(drift[s], kick[s])
        pos1, vel1, _, _ = box.get_state()
        box.close()
        assert np.array_equal(pos, pos1) and np.array_equal(vel, vel1), f"box {b} differs from the box alone"
    ens.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_FIXED])
def test_ensemble_shared_pair_law_tracks_single_boxes(mode):
    """Boxes of one configuration (seeds apart) share one pair law, which the
    short range then takes as a kernel parameter instead of from each box's
    descriptor; forces and graph-replayed steps still equal each box alone,
    bit for bit."""
    ics_, cfgs = make([(16, 32, 60.0, s) for s in (21, 22, 23)], mode)
    ens = Ensemble(cfgs)
    for b, ic in enumerate(ics_):
        ens.set_state(b, ic.pos)
    ens.forces()
    for b, (ic, c) in enumerate(zip(ics_, cfgs)):
        _, _, app, apm = ens.get_state(b)
        box = Box(BoxConfig(**{**c.__dict__, "cell_grid": ens.plan(b)[0]}))
        box.set_state(ic.pos)
        box.forces()
        _, _, app1, apm1 = box.get_state()
        box.close()
        assert np.array_equal(app, app1), f"box {b}: short range differs from the box alone"
        assert np.array_equal(apm, apm1), f"box {b}: PM differs from the box alone"
    ens.close()

    ens = Ensemble(cfgs)
    for b, ic in enumerate(ics_):
        ens.set_state(b, ic.pos, ic.canonical_velocity())
    a, drift, kick = fixed_step_schedule(ics_[0].a, 0.05, 3)
    for s in range(4):  # the first call captures the graph, the rest replay it
        ens.step(drift[s], kick[s])
    ens.sync()
    for b, (ic, c) in enumerate(zip(ics_, cfgs)):
        pos, vel, _, _ = ens.get_state(b)
        box = Box(BoxConfig(**{**c.__dict__, "cell_grid": ens.plan(b)[0]}))
        box.set_state(ic.pos, ic.canonical_velocity())
        for s in range(4):
            box.step(drift[s], kick[s])
        pos1, vel1, _, _ = box.get_state()
        box.close()
        assert np.array_equal(pos, pos1) and np.array_equal(vel, vel1), f"box {b} differs from the box alone"
    ens.close()


def test_ensemble_reshape_carries_state():
    """Boxes kept across a reshape (reordered, one dropped, one added, the
    particle count growing past the arrays' capacity) continue exactly as
    single boxes stepped alone."""
    ics_, cfgs = make(SPECS, MODE_FIXED)
    a, drift, kick = fixed_step_schedule(ics_[0].a, 0.05, 5)
    ens = Ensemble(cfgs[:2])
    for b in range(2):
        ens.set_state(b, ics_[b].pos, ics_[b].canonical_velocity())
    for s in range(3):
        ens.step(drift[s], kick[s])
    before = [ens.get_state(b)[:2] for b in range(2)]
    # new layout: box 1 first, then the two new boxes (more particles than before); box 0 leaves
    ens.reshape([cfgs[1], cfgs[2], cfgs[3]], [1, -1, -1])
    pos, vel, _, _ = ens.get_state(0)
    assert np.array_equal(pos, before[1][0]) and np.array_equal(vel, before[1][1])
    for b, k in ((1, 2), (2, 3)):
        ens.set_state(b, ics_[k].pos, ics_[k].canonical_velocity())
    for s in range(3, 6):
        ens.step(drift[s], [kick[s]] * 3)
    ens.sync()
    # box 1 ran steps 0..5, boxes 2 and 3 ran steps 3..5 from their ICs
    for b, k, steps in ((0, 1, range(6)), (1, 2, range(3, 6)), (2, 3, range(3, 6))):
        pos, vel, _, _ = ens.get_state(b)
        box = Box(BoxConfig(**{**cfgs[k].__dict__, "cell_grid": ens.plan(b)[0]}))
        box.set_state(ics_[k].pos, ics_[k].canonical_velocity())
        for s in steps:
            box.step(drift[s], kick[s])
        pos1, vel1, _, _ = box.get_state()
        box.close()
        assert np.array_equal(pos, pos1) and np.array_equal(vel, vel1), f"box {b} differs after the reshape"
    ens.close()
