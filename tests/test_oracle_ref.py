"""The oracle's C restatement against the reference's own CPU code.

The reference's CPU force path (gravlist.cpp, pm_periodic.c, driftfac.c) is
compiled from its sources by oracle/Makefile into oracle/_ref/.  These tests
need the reference sources and are skipped where they are absent.
"""
import os

import numpy as np
import pytest

import oracle
from cuco_gb300 import ics
from conftest import rms_rel

pytestmark = pytest.mark.skipif(not oracle.reference_available(),
                                reason="reference sources not present")


def setup_ref(pmgrid, n_side, box_mpc, seed, frac=0.03):
    ic = ics.zeldovich(n_side, box_mpc, 49.0, seed)
    ref = oracle.Reference(pmgrid)
    eps = float(np.float32(frac * ic.boxsize / n_side))
    ref.begrun(ic, soft_comoving=eps)
    return ic, ref


@pytest.mark.parametrize("pmgrid,n_side,box", [(32, 16, 50.0), (64, 32, 100.0), (128, 32, 100.0),
                                                (512, 32, 100.0)])
def test_port_forces_bit_exact(port, pmgrid, n_side, box):
    """Short range and PM of the restatement equal the reference's own, bit for
    bit, from the smallest mesh to the 512 mesh (the reference built with
    that PMGRID; its PM takes ~40 s there on one core)."""
    ic, ref = setup_ref(pmgrid, n_side, box, seed=pmgrid)
    pos = ref.get()[0]
    app = ref.pp(1)
    apm = ref.pm()
    p = oracle.reference_params(ic.boxsize, ic.mass, ref.G, pmgrid, ref.softening)
    assert p.asmth == np.float32(ref.asmth) and p.rcut == np.float32(ref.rcut)
    assert np.array_equal(port.pp(pos, p, pmgrid, 4), app)
    assert np.array_equal(port.pm(pos, p, pmgrid, 4), apm)


@pytest.mark.skipif(os.environ.get("CUCO_ORACLE_LARGE_MESH") != "1",
                    reason="~7 minutes and ~30 GB of host memory; set CUCO_ORACLE_LARGE_MESH=1")
def test_port_forces_bit_exact_mesh_1024(port):
    """The 1024 mesh (the 512^3 workload's): the restatement's PM and short
    range equal the reference built with PMGRID 1024, bit for bit."""
    test_port_forces_bit_exact(port, 1024, 32, 100.0)


def test_port_pp_threads_and_targets(port):
    ic, ref = setup_ref(32, 16, 50.0, seed=3)
    pos = ref.get()[0]
    p = oracle.reference_params(ic.boxsize, ic.mass, ref.G, 32, ref.softening)
    ref.pp(4)  # the harness's threaded split of force_evaluate_shortrange
    app4 = ref.get()[2]
    assert np.array_equal(app4, ref.pp(1))
    sub = np.array([0, 17, 999, 4095])
    assert np.array_equal(port.pp_targets(pos, sub, p, 32, 2), app4[sub])


def test_drift_tables_and_factors(port):
    ic, ref = setup_ref(32, 16, 50.0, seed=5)
    d_ref, k_ref = ref.tables()
    a0 = float(np.float32(ic.a))
    d64, k64 = port.drift_tables(a0, 1.0, 0.3, 0.7, ref.lib.cref_hubble())
    # the reference stores float tables; the FP64 ones round to them
    assert np.max(np.abs(d64.astype(np.float32).view(np.int32) - d_ref.view(np.int32))) <= 1
    assert np.max(np.abs(k64.astype(np.float32).view(np.int32) - k_ref.view(np.int32))) <= 1
    l0, l1, tbi = np.log(a0), 0.0, ref.timebase_interval
    for t0, t1 in [(0, 1 << 20), (3, 1 << 27), (1 << 27, 1 << 28)]:
        # same arithmetic on the reference's float tables gives its exact factors
        assert port.table_factor(d_ref.astype(np.float64), l0, l1, tbi, t0, t1) == \
            ref.lib.cref_drift_factor(t0, t1)
        assert port.table_factor(k_ref.astype(np.float64), l0, l1, tbi, t0, t1) == \
            ref.lib.cref_kick_factor(t0, t1)


def test_simparam_matches_reference(port):
    ic, ref = setup_ref(64, 16, 50.0, seed=6)
    sp = ref.simparam()
    assert np.array_equal(sp[:1000], port.shortrange_table())
    boxsize, boxhalf, to_grid_fac, rcut, rcut2, asmth, asmthfac, mass, G = sp[1000:]
    assert to_grid_fac == np.float32(np.float32(64) / np.float32(ic.boxsize))
    assert rcut == np.float32(ref.rcut) and asmth == np.float32(ref.asmth)
    assert asmthfac == np.float32(0.5 / np.float64(np.float32(ref.asmth)) * (1000 / 3.0))
    assert mass == np.float32(ic.mass) and boxsize == np.float32(ic.boxsize)


def test_keys_rule_and_sort(port):
    rng = np.random.default_rng(0)
    L = np.float32(256000.0)
    pos = rng.uniform(0, L, size=(50000, 3)).astype(np.float32)
    pos[:3] = np.nextafter(L, np.float32(0))
    G = 64
    gf = np.float32(np.float32(G) / L)
    keys = port.keys(pos, gf, G)
    c = np.minimum((gf * pos).astype(np.float32).astype(np.int64), G - 1)  # float32 product, truncated
    assert np.array_equal(keys, ((c[:, 0] * G + c[:, 1]) * G + c[:, 2]).astype(np.uint32))
    sk, perm = port.stable_sort(keys, G ** 3)
    assert np.array_equal(perm, np.argsort(keys, kind="stable").astype(np.uint32))
    assert np.array_equal(sk, keys[perm])
    start, end = port.cell_bounds(sk, G ** 3)
    u, first, counts = np.unique(sk, return_index=True, return_counts=True)
    assert np.array_equal(start[u], first) and np.array_equal(end[u], first + counts)
    empty = np.setdiff1d(np.arange(G ** 3), u)
    assert np.all(start[empty] == 0xFFFFFFFF)


def test_reference_method_floor_vs_ewald(port):
    """The reference's own PM + short-range force against the FP64 Ewald sum:
    the method floor the engine's errors are read against (16^3, PMGRID 32)."""
    ic, ref = setup_ref(32, 16, 50.0, seed=8)
    pos = ref.get()[0]
    tot = ref.pp(1).astype(np.float64) + ref.pm().astype(np.float64)
    rng = np.random.default_rng(1)
    sub = rng.choice(ic.n, 512, replace=False)
    ew = port.ewald(pos.astype(np.float64), float(np.float32(ic.mass)), ref.G, float(np.float32(ic.boxsize)),
                    ref.softening, pos[sub].astype(np.float64), 8)
    err = rms_rel(tot[sub], ew)
    print(f"reference P3M vs Ewald rms {err:.3e}")
    assert err < 5e-2
