"""The fixed-point precision form (CUCO_MODE_FIXED) on the GPU.

Positions are uint32 per axis in units of L / 2^32.  What is integer work is
checked bit for bit against numpy: the float -> fixed conversion, the drift
(one rounding of the displacement to the grid, then a modular add, so the
periodic wrap is exact), the cell keys floor(x * G / 2^32) and the stable sort
permutation.  Forces are compared with the reference's own FP64 path (the
oracle) at the tolerance the reduced-precision form must meet: rms relative
error <= 1e-3.
"""
import numpy as np
import pytest

import oracle
from cuco_gb300 import Box, BoxConfig, ics
from cuco_gb300.engine import MODE_FIXED
from helpers import clustered, softening_h, zeldovich
from conftest import rms_rel

pytestmark = pytest.mark.gpu

TOL_FIXED = 1e-3
TWO32 = 2.0 ** 32


def to_fixed(pos, L):
    return (np.rint(pos.astype(np.float64) * (TWO32 / L)).astype(np.int64) & 0xFFFFFFFF).astype(np.uint32)


def from_fixed(u, L):
    return (u.astype(np.float64) * (L / TWO32)).astype(np.float32)


def fixed_box(n, L, mass, M, G, soft):
    return Box(BoxConfig(n=n, pm_grid=M, cell_grid=G, boxsize=L, mass=mass, G=ics.G_INTERNAL,
                         softening=soft, mode=MODE_FIXED))


def test_fixed_state_conversion_and_round_trip():
    ic = zeldovich(16, 50.0)
    box = fixed_box(ic.n, ic.boxsize, ic.mass, 32, 16, softening_h(ic.boxsize, 16))
    pos = ic.pos.copy()
    pos[:5, 0] = [-1e-3, ic.boxsize, ic.boxsize + 10.0, -ic.boxsize * 0.25, 0.0]  # wrapped on entry
    box.set_state(pos, ic.vel)
    u = box.get_state_fixed()
    assert np.array_equal(u, to_fixed(pos, ic.boxsize))
    back = box.get_state()[0]
    assert np.array_equal(back, from_fixed(u, ic.boxsize))
    # exact fixed-point I/O
    rng = np.random.default_rng(2)
    u2 = rng.integers(0, 2 ** 32, size=(ic.n, 3), dtype=np.uint64).astype(np.uint32)
    box.set_state_fixed(u2, ic.vel)
    assert np.array_equal(box.get_state_fixed(), u2)
    box.close()


@pytest.mark.parametrize("G", [16, 12])
def test_fixed_keys_and_sort_bit_exact(port, G):
    rng = np.random.default_rng(G)
    n = 50000
    L = 20000.0
    u = rng.integers(0, 2 ** 32, size=(n, 3), dtype=np.uint64).astype(np.uint32)
    u[:64] = u[0]  # equal keys: stability
    u[64:70] = [0xFFFFFFFF, 0, 0x80000000]  # the grid's edges
    box = fixed_box(n, L, 1.0, 32, G, 10.0)
    box.set_state_fixed(u)
    box.forces(pm=False, pp=False)
    keys, perm, _, _ = box.debug()
    k = (u.astype(np.uint64) * np.uint64(G)) >> np.uint64(32)
    key = ((k[:, 0] * G + k[:, 1]) * G + k[:, 2]).astype(np.uint32)
    order = np.argsort(key, kind="stable")
    assert np.array_equal(perm, order.astype(np.uint32))
    assert np.array_equal(keys, key[order])
    box.close()


def test_fixed_drift_exact_and_periodic():
    n = 4096
    L = 1000.0
    rng = np.random.default_rng(7)
    u = rng.integers(0, 2 ** 32, size=(n, 3), dtype=np.uint64).astype(np.uint32)
    u[:16] = 0xFFFFFF00  # next to the upper face: these wrap
    vel = rng.normal(0, 300.0, size=(n, 3)).astype(np.float32)
    vel[:16] = 500.0
    box = fixed_box(n, L, 1e-6, 64, 16, 1.0)
    box.set_state_fixed(u, vel)
    drift = 0.0123
    box.step(drift, 0.0, 0.0)
    got = box.get_state_fixed()
    upt = np.float32(drift * TWO32 / L)
    disp = np.rint((vel * upt).astype(np.float32).astype(np.float64)).astype(np.int64)
    want = ((u.astype(np.int64) + disp) & 0xFFFFFFFF).astype(np.uint32)
    assert np.array_equal(got, want)
    assert np.all(got[:16] < u[:16])  # crossed the face, came back at the bottom
    box.close()


@pytest.mark.parametrize("kind", ["zeldovich", "clustered"])
def test_fixed_forces_vs_reference_path(port, kind):
    if kind == "zeldovich":
        ic = zeldovich(32, 100.0)
        pos, L, mass = ic.pos, ic.boxsize, ic.mass
    else:
        L, mass = 100000.0, 100.0
        pos = clustered(30000, L, seed=5)
    n = pos.shape[0]
    M, G = 64, 16
    soft = softening_h(L, 32)
    box = fixed_box(n, L, mass, M, G, soft)
    box.set_state(pos)
    box.forces()
    _, _, app, apm = box.get_state()
    # the oracle sees the positions the box holds (fixed point rounded to float)
    pf = from_fixed(to_fixed(pos, L), L)
    p = oracle.reference_params(L, mass, ics.G_INTERNAL, M, soft)
    ref_pp = port.pp(pf, p, G, 8)
    ref_pm = port.pm(pf, p, M, 8)
    e_pp, e_pm = rms_rel(app, ref_pp), rms_rel(apm, ref_pm)
    e_tot = rms_rel(app + apm, ref_pp + ref_pm)
    print(f"fixed {kind}: pp {e_pp:.2e} pm {e_pm:.2e} total {e_tot:.2e}")
    assert e_pp < TOL_FIXED and e_pm < TOL_FIXED and e_tot < TOL_FIXED
    box.close()


def test_fixed_step_matches_plain_step():
    """Three full steps of the fixed-point form stay within the reduced-precision
    bar of the plain form's trajectory (velocities after three kicks)."""
    ic = zeldovich(32, 100.0)
    soft = softening_h(ic.boxsize, 32)
    from cuco_gb300 import fixed_step_schedule
    a, drift, kick = fixed_step_schedule(ic.a, 0.05, 3)
    out = []
    for mode in (0, MODE_FIXED):
        box = Box(BoxConfig(n=ic.n, pm_grid=64, cell_grid=16, boxsize=ic.boxsize, mass=ic.mass,
                            G=ics.G_INTERNAL, softening=soft, mode=mode))
        box.set_state(ic.pos, ic.canonical_velocity())
        for s in range(3):
            box.step(drift[s], kick[s])
        out.append(box.get_state())
        box.close()
    (p0, v0, _, _), (p1, v1, _, _) = out
    v_init = ic.canonical_velocity()
    dv = rms_rel(v1 - v_init, v0 - v_init)  # the fixed form's velocity change against the plain one's
    dx = np.abs(p1 - p0)
    dx = np.minimum(dx, ic.boxsize - dx)
    print(f"fixed vs plain after 3 steps: dv/|v change| {dv:.2e}, max dx {dx.max():.2e}")
    assert dv < TOL_FIXED
    assert dx.max() < 1e-4 * ic.boxsize
