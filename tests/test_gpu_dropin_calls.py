"""Reference-named drop-in entry points called one at a time, as a host program
that keeps part of the reference's own code would call them:
copyPosToDevice / copyAccelFromDevice (gravlist.cu:56-83), do_box_wrapping
(predict.c:24-41), long_range_force (longrange.c:14-22) and get_timestep
(timestep.c:96-138), each against a restatement of the reference's rule or
the oracle."""
import ctypes
import math

import numpy as np
import pytest

import oracle
from cuco_gb300 import ics
from conftest import rms_rel
from dropin_host import DropIn
from helpers import zeldovich

pytestmark = pytest.mark.gpu

NS, BOX, M = 16, 50.0, 32


@pytest.fixture()
def dropin():
    ic = zeldovich(NS, BOX, seed=21)
    eps = 0.03 * ic.boxsize / NS
    return ic, DropIn(ic.pos, ic.canonical_velocity(), ic.mass, ic.boxsize, ic.a, M, 0, eps)


def _dev_array(lib, name, n):
    p = ctypes.c_void_p.in_dll(lib, name).value
    assert p, name + " not set by linklist_init"
    out = np.empty((n, 4), dtype=np.float32)
    lib.copyArrayFromDevice(out.ctypes.data, ctypes.c_void_p(p), out.nbytes)
    return p, out


def test_copy_pos_to_device_and_accel_from_device(dropin):
    ic, d = dropin
    lib, n = d.lib, d.n
    rng = np.random.default_rng(5)
    new_pos = rng.uniform(0, ic.boxsize, (n, 3)).astype(np.float32)
    d._raw()[:, 0:3] = new_pos
    lib.copyPosToDevice()
    _, dev_pos = _dev_array(lib, "dOldPos", n)
    assert np.array_equal(dev_pos[:, :3], new_pos)
    # a known acceleration field in dGravAccel comes back into P[].GravAccel
    acc = np.zeros((n, 4), dtype=np.float32)
    acc[:, :3] = rng.normal(0, 1e3, (n, 3))
    p_acc, _ = _dev_array(lib, "dGravAccel", n)
    lib.copyArrayToDevice(ctypes.c_void_p(p_acc), acc.ctypes.data, 0, acc.nbytes)
    before = d.field("Pos")
    lib.copyAccelFromDevice()
    assert np.array_equal(d.field("GravAccel"), acc[:, :3])
    assert np.array_equal(d.field("Pos"), before)  # nothing else written


def _wrap_reference(x, L):
    """predict.c:33-39: while loops in float storage with a double box size."""
    x = x.astype(np.float32).copy()
    for _ in range(8):
        lo = x < 0
        x[lo] = (x[lo].astype(np.float64) + L).astype(np.float32)
        hi = x >= L
        x[hi] = (x[hi].astype(np.float64) - L).astype(np.float32)
    return x


def test_do_box_wrapping(dropin):
    ic, d = dropin
    L = float(np.float32(ic.boxsize))
    pos = ic.pos.astype(np.float32).copy()
    rng = np.random.default_rng(6)
    shift = rng.integers(-2, 3, size=pos.shape).astype(np.float32) * np.float32(L)
    moved = (pos + shift).astype(np.float32)
    moved[0] = [-0.0, L, -1e-7]  # the edges: -0 stays, L wraps to 0, tiny negatives
    d._raw()[:, 0:3] = moved
    d.lib.do_box_wrapping()
    got = d.field("Pos")
    assert np.array_equal(got, _wrap_reference(moved, L))
    assert (got >= 0).all() and (got < L).all()


def test_long_range_force_vs_oracle(dropin, port):
    ic, d = dropin
    # stale values must be replaced, not added to (longrange.c:17-19 zeroes GravPM)
    d._raw()[:, 10:13] = 1e9
    d.lib.long_range_force()
    p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, M, d.All.ForceSoftening)
    ref = port.pm(d.field("Pos"), p, M, 4)
    assert rms_rel(d.field("GravPM"), ref) < 1e-4


def _get_timestep_reference(al, acc_pp, acc_pm):
    """timestep.c:96-138 with the factors advance_and_find_timesteps sets (11-24)."""
    a = al.Time
    f32 = np.float32
    # C's float arithmetic where timestep.c mixes only floats and ints:
    # 1 / (All.Time * All.Time) and 1 - Omega0 - OmegaLambda
    fac1 = float(f32(1) / (f32(a) * f32(a)))
    curv = float(f32(1) - f32(al.Omega0) - f32(al.OmegaLambda))
    hubble_a = al.Hubble * math.sqrt(al.Omega0 / (a * a * a) + curv / (a * a) + al.OmegaLambda)
    acc = fac1 * acc_pp.astype(np.float64) + fac1 * acc_pm.astype(np.float64)
    ac = np.sqrt((acc ** 2).sum(axis=1))
    ac[ac == 0] = 1e-30
    dt = np.sqrt(2 * al.ErrTolIntAccuracy * a * al.SofteningTable / ac) * hubble_a
    dt = np.minimum(dt, al.MaxSizeTimestep)
    dt = np.maximum(dt, al.MinSizeTimestep)
    return (dt / al.Timebase_interval).astype(np.int64)


def test_get_timestep_direct_calls(dropin):
    ic, d = dropin
    d.lib.compute_accelerations()
    # a spread of accelerations so some particles get steps below the cap
    scale = np.geomspace(1.0, 1e6, d.n).astype(np.float32)
    d._raw()[:, 7:10] *= scale[:, None]
    ref = _get_timestep_reference(d.All, d.field("GravAccel"), d.field("GravPM"))
    # only particles whose step is a valid one: get_timestep exits the process
    # on a zero step, as timestep.c:128-135 does
    ok = np.flatnonzero((ref > 0) & (ref < (1 << 28)))
    assert ok.size > d.n // 2
    idx = ok[np.linspace(0, ok.size - 1, 64).astype(int)]
    got = np.array([d.lib.get_timestep(int(i)) for i in idx])
    assert np.array_equal(got, ref[idx])
    assert len(set(got.tolist())) > 4
