"""The GPU path against fixtures produced by the reference's own CPU code
(tests/golden/make_golden.py): forces at the IC (16^3 with PMGRID 32, and the
small workload's 32^3 box with PMGRID 64 on a subsample of targets), and
passes of the reference's run loop driven through the drop-in C ABI."""
import os

import numpy as np
import pytest

from cuco_gb300 import Box, BoxConfig
from conftest import rms_rel
from dropin_host import DropIn

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_n16_pm32.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(FIX))


def test_restatement_on_this_host_vs_fixtures(port, gold):
    """The oracle's restatement - the checker of the other GPU tests - on the
    host these tests run on, where the reference's sources are absent: its
    short range and PM equal the reference-made fixtures bit for bit (this
    test itself uses no GPU)."""
    import oracle
    for g, tg in ((gold, None), (dict(np.load(os.path.join(os.path.dirname(FIX), "ref_n32_pm64.npz"))), "targets")):
        p = oracle.OpParams(float(g["boxsize"]), float(np.float32(g["mass"])), float(g["G"]),
                            float(g["asmth"]), float(g["rcut"]), float(g["softening"]))
        M = int(g["pmgrid"])
        if tg is None:
            assert np.array_equal(port.pp(g["pos"], p, M, 4), g["acc_pp"])
            assert np.array_equal(port.pm(g["pos"], p, M, 4), g["acc_pm"])
        else:
            assert np.array_equal(port.pp_targets(g["pos"], g[tg], p, M, 4), g["acc_pp"])
            assert np.array_equal(port.pm(g["pos"], p, M, 4)[g[tg]], g["acc_pm"])


@pytest.mark.parametrize("cell_grid", [32, 16, 8])
def test_forces_vs_reference_fixture(gold, cell_grid):
    M = int(gold["pmgrid"])
    n = gold["pos"].shape[0]
    box = Box(BoxConfig(n=n, pm_grid=M, cell_grid=cell_grid, boxsize=float(gold["boxsize"]),
                        mass=float(gold["mass"]), G=float(gold["G"]), softening=float(gold["softening"]),
                        asmth=float(gold["asmth"]), rcut=float(gold["rcut"])))
    box.set_state(gold["pos"], gold["vel"])
    box.forces()
    _, _, app, apm = box.get_state()
    e_pp, e_pm = rms_rel(app, gold["acc_pp"]), rms_rel(apm, gold["acc_pm"])
    print(f"G={cell_grid}: pp {e_pp:.2e} pm {e_pm:.2e}")
    assert e_pp < 1e-4 and e_pm < 1e-4
    box.close()


@pytest.mark.parametrize("cell_grid", [64, 16])
def test_small_workload_forces_vs_reference_fixture(cell_grid):
    """The small workload's box (32^3, L = 100 Mpc/h, M = 64) against the
    reference's own forces on the fixture's 4096 targets."""
    g = dict(np.load(os.path.join(os.path.dirname(FIX), "ref_n32_pm64.npz")))
    M, tg = int(g["pmgrid"]), g["targets"]
    box = Box(BoxConfig(n=g["pos"].shape[0], pm_grid=M, cell_grid=cell_grid, boxsize=float(g["boxsize"]),
                        mass=float(g["mass"]), G=float(g["G"]), softening=float(g["softening"]),
                        asmth=float(g["asmth"]), rcut=float(g["rcut"])))
    box.set_state(g["pos"])
    box.forces()
    _, _, app, apm = box.get_state()
    box.close()
    e_pp, e_pm = rms_rel(app[tg], g["acc_pp"]), rms_rel(apm[tg], g["acc_pm"])
    print(f"32^3 M=64 G={cell_grid}: pp {e_pp:.2e} pm {e_pm:.2e}")
    assert e_pp < 1e-4 and e_pm < 1e-4


@pytest.mark.parametrize("mirror", ["0", "1"])
def test_dropin_run_loop_vs_reference(gold, mirror, monkeypatch):
    # "1": P[] copied whole to a device mirror around each call; "0": the
    # kernels work on the host P[] in place where the device allows it
    monkeypatch.setenv("CUCO_DROPIN_MIRROR", mirror)
    M = int(gold["pmgrid"])
    d = DropIn(gold["pos"], gold["vel"], float(gold["mass"]), float(gold["boxsize"]),
               float(gold["a_begin"]), M, 0, float(gold["eps"]))
    assert d.All.Asmth == np.float32(gold["asmth"]) and d.All.Rcut == np.float32(gold["rcut"])
    tis = []
    for _ in range(3):
        tis.append(d.run_pass())
        # the device-side minimum equals the host scan of run.c:35-40
        assert d.lib.cuco_dropin_min_ti_endstep() == int(d.timeline()[1].min())
    assert tis == list(gold["run_ti_current"])
    beg, end = d.timeline()
    assert np.array_equal(beg, gold["run_ti_beg"]) and np.array_equal(end, gold["run_ti_end"])
    assert [d.All.PM_Ti_begstep, d.All.PM_Ti_endstep, d.All.Ti_Current] == list(gold["run_pm_ti"])
    assert rms_rel(d.field("GravAccel"), gold["run_acc_pp"]) < 1e-4
    assert rms_rel(d.field("GravPM"), gold["run_acc_pm"]) < 1e-4
    assert rms_rel(d.field("Vel"), gold["run_vel"]) < 1e-4
    dx = np.abs(d.field("Pos") - gold["run_pos"])
    dx = np.minimum(dx, float(gold["boxsize"]) - dx)
    assert dx.max() < 1e-4 * float(gold["boxsize"])


@pytest.fixture(scope="module")
def gold_mixed():
    return dict(np.load(os.path.join(os.path.dirname(FIX), "ref_n16_pm32_mixed.npz")))


def test_dropin_run_loop_individual_timesteps(gold_mixed):
    """Eight passes of the reference's run loop on a box whose particles take
    three different power-of-two steps (timestep.c:11-94): the integer
    timeline of every particle and of the PM step, the velocities (kicked
    only when a particle is active), the positions (drifted every pass), and
    the short-range force of the particles active at the last pass.  The
    reference's CPU loop computes the short range for active particles only
    (gravlist.cpp:208) and the GPU path for all (as gravity_linklist_cuda
    does); an inactive particle's stored force is not used before it is
    recomputed, so only the active ones are compared."""
    g = gold_mixed
    M = int(g["pmgrid"])
    d = DropIn(g["pos"], g["vel"], float(g["mass"]), float(g["boxsize"]), float(g["a_begin"]), M, 0,
               float(g["eps"]), errtol=float(g["errtol"]), max_dloga=float(g["max_dloga"]))
    tis = [d.run_pass() for _ in range(len(g["run_ti_current"]))]
    assert tis == list(g["run_ti_current"])
    beg, end = d.timeline()
    steps = np.unique(g["run_ti_end"] - g["run_ti_beg"])
    assert steps.size >= 3  # the fixture really mixes step sizes
    assert np.array_equal(beg, g["run_ti_beg"]) and np.array_equal(end, g["run_ti_end"])
    assert [d.All.PM_Ti_begstep, d.All.PM_Ti_endstep, d.All.Ti_Current] == list(g["run_pm_ti"])
    active = beg == tis[-1]
    assert 0 < active.sum() < d.n
    assert rms_rel(d.field("GravAccel")[active], g["run_acc_pp"][active]) < 1e-4
    assert rms_rel(d.field("GravPM"), g["run_acc_pm"]) < 1e-4
    assert rms_rel(d.field("Vel"), g["run_vel"]) < 1e-4
    dx = np.abs(d.field("Pos") - g["run_pos"])
    dx = np.minimum(dx, float(g["boxsize"]) - dx)
    assert dx.max() < 1e-4 * float(g["boxsize"])
