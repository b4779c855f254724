"""Force error of the two forms against the reference's FP64 path on the
bench workload's mid size (128^3, L = 256 Mpc/h, M = 256, G = 64), at the
start (z = 49) and after the whole 200-step run to z = 0 (strongly
clustered), on a seeded 4096-particle subsample of targets.

The precision form (uint32 fixed-point positions, FP32 pair force and PM,
compensated reduction) must stay within rms 1e-3 of the FP64 path; the plain
form within 1e-4.  Both are printed side by side, with the median and 99th
percentile of the per-particle relative error beside each rms.  The state at z = 0 comes
from the plain form's own run; both forms then evaluate forces on that same
state (the fixed-point form rounds it to its 2^-32 L grid, and the oracle sees
that rounding).
"""
import numpy as np
import pytest

import oracle
from cuco_gb300 import Box, BoxConfig, fixed_step_schedule, ics
from cuco_gb300.engine import MODE_FIXED
from conftest import err_stats

pytestmark = pytest.mark.gpu

N_SIDE, BOX_MPC, M, G, Z0, SEED, STEPS = 128, 256.0, 256, 64, 49.0, 12345, 200
NSUB = 4096


def rounded_to_fixed(pos, L):
    u = (np.rint(pos.astype(np.float64) * (2.0 ** 32 / L)).astype(np.int64) & 0xFFFFFFFF)
    return (u.astype(np.float64) * (L / 2.0 ** 32)).astype(np.float32)


@pytest.fixture(scope="module")
def states():
    ic = ics.zeldovich(N_SIDE, BOX_MPC, Z0, SEED)
    soft = float(np.float32(2.8 * np.float32(0.025 * ic.boxsize / N_SIDE)))
    box = Box(BoxConfig(n=ic.n, pm_grid=M, cell_grid=G, boxsize=ic.boxsize, mass=ic.mass,
                        G=ics.G_INTERNAL, softening=soft))
    box.set_state(ic.pos, ic.canonical_velocity())
    a, drift, kick = fixed_step_schedule(ic.a, 1.0, STEPS)
    for s in range(STEPS + 1):
        box.step(drift[s], kick[s])
    late = box.get_state()[0]
    box.close()
    return ic, soft, {"z49": ic.pos, "z0": late}


@pytest.mark.parametrize("when", ["z49", "z0"])
def test_forms_vs_fp64_path(port, states, when):
    ic, soft, st = states
    L, pos = ic.boxsize, st[when]
    sub = np.sort(np.random.default_rng(4096).choice(ic.n, NSUB, replace=False))
    p = oracle.reference_params(L, ic.mass, ics.G_INTERNAL, M, soft)
    errs = {}
    for mode, name in ((0, "plain"), (MODE_FIXED, "precision")):
        box = Box(BoxConfig(n=ic.n, pm_grid=M, cell_grid=G, boxsize=L, mass=ic.mass, G=ics.G_INTERNAL,
                            softening=soft, mode=mode))
        box.set_state(pos)
        box.forces()
        _, _, app, apm = box.get_state()
        box.close()
        pref = rounded_to_fixed(pos, L) if mode else pos
        ref_pp = port.pp_targets(pref, sub, p, M, 16)
        ref_pm = port.pm(pref, p, M, 16)[sub]
        errs[name] = (err_stats(app[sub], ref_pp), err_stats(apm[sub], ref_pm),
                      err_stats(app[sub] + apm[sub], ref_pp + ref_pm))
    for name, es in errs.items():
        print(f"{when} {name:9s}: " + "  ".join(
            f"{part} {e['rms']:.2e}/{e['median']:.2e}/{e['p99']:.2e}" for part, e in zip(("pp", "pm", "total"), es))
            + "  (rms/median/p99)")
    assert max(e["rms"] for e in errs["plain"]) < 1e-4
    assert max(e["rms"] for e in errs["precision"]) < 1e-3


@pytest.mark.parametrize("when", ["z49", "z0"])
def test_forms_vs_ewald(port, states, when):
    """Total force of both forms and of the reference method (the floor)
    against the FP64 Ewald oracle on the same 4096-particle subsample."""
    from test_gpu_ewald import check_against_floor, ewald_table, table_line
    ic, soft, st = states
    sub = np.sort(np.random.default_rng(4096).choice(ic.n, NSUB, replace=False))
    t = ewald_table(port, st[when], ic, soft, M, sub)
    print(table_line(f"EWALD 128^3 M=256 {when}", t))
    check_against_floor(t)
