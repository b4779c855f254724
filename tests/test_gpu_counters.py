"""The engine's instrumentation: the in-range pair count of the short range
and the per-phase device times.

The pair count (r^2 <= rcut^2, the self pair excluded) is compared with a
brute-force count in double precision over all minimum-image pairs; the two
may differ only for pairs within rounding of the cut.  The phase times of a
run of steps are non-negative and tile the timed total (the PM beside the
sort and the reorder).
"""
import numpy as np
import pytest

from cuco_gb300 import Box, BoxConfig, fixed_step_schedule, ics
from helpers import clustered, softening_h, zeldovich

pytestmark = pytest.mark.gpu


def brute_pairs(pos, L, rcut):
    p = pos.astype(np.float64)
    total = 0
    for i in range(0, p.shape[0], 512):
        d = p[i:i + 512, None, :] - p[None, :, :]
        d -= L * np.round(d / L)
        r2 = (d * d).sum(-1)
        total += int(np.count_nonzero(r2 <= rcut * rcut))
    return total - p.shape[0]  # the self pairs


@pytest.mark.parametrize("kind", ["zeldovich", "clustered"])
def test_pair_count_matches_brute_force(kind):
    if kind == "zeldovich":
        ic = zeldovich(16, 50.0)
        pos, L, mass = ic.pos, ic.boxsize, ic.mass
    else:
        L, mass = 50000.0, 1.0
        pos = clustered(4000, L, seed=8)
    box = Box(BoxConfig(n=pos.shape[0], pm_grid=32, cell_grid=8, boxsize=L, mass=mass, G=ics.G_INTERNAL,
                        softening=softening_h(L, 16)))
    box.set_state(pos)
    box.count_pairs(True)
    box.pair_count(reset=True)
    box.forces(pm=False, pp=True)
    got = box.pair_count()
    want = brute_pairs(box.get_state()[0], L, float(box.c.rcut))
    print(f"{kind}: pairs {got} brute force {want}")
    assert abs(got - want) <= max(2, want // 100000)
    box.count_pairs(False)
    box.pair_count(reset=True)
    box.forces(pm=False, pp=True)
    assert box.pair_count() == 0  # not counted unless enabled
    box.close()


def test_phase_totals_add_up():
    ic = zeldovich(32, 100.0)
    box = Box(BoxConfig(n=ic.n, pm_grid=64, cell_grid=16, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                        softening=softening_h(ic.boxsize, 32)))
    box.set_state(ic.pos, ic.canonical_velocity())
    a, drift, kick = fixed_step_schedule(ic.a, 0.05, 5)
    box.enable_timing(True)
    for s in range(5):
        box.step(drift[s], kick[s])
    t = box.phase_totals()
    box.close()
    parts = [v for k, v in t.items() if k != "total"]
    assert all(v >= 0.0 for v in parts)
    assert t["total"] > 0.0
    # Each step is drift+keys, then two branches side by side (sort and
    # reorder; the PM on its own stream), then the short range.  Summed over
    # steps, the longer branch lies between the larger branch total and the
    # sum of both; the tolerance covers event granularity.
    serial = t["drift+keys"] + t["shortrange"]
    a = t["sort"] + t["reorder"]
    b = t["pm_deposit"] + t["pm_fft"] + t["pm_interp"]
    tol = 0.05 * t["total"] + 0.05
    assert serial + max(a, b) <= t["total"] + tol
    assert t["total"] <= serial + a + b + tol
