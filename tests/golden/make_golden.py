"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own CPU force path (compiled from its sources into
oracle/_ref/ by oracle/Makefile, see oracle/ref_harness.c) on a seeded 16^3
Zel'dovich box (L = 50 Mpc/h, z = 49, PMGRID = 32) and stores:
  pos, vel        state after init() (velocities scaled by a^{3/2}, init.c:30)
  acc_pp          gravity_linklist() short-range force (gravlist.cpp:195-338)
  acc_pm          long_range_force() PM force (longrange.c:14-22)
  drift, kick     the float drift/kick tables (driftfac.c:14-42)
  factors         get_drift_factor / get_gravkick_factor at fixed (t0, t1)
  run_*           state after 3 passes of the reference run loop with the CPU
                  short range (run.c:11-20, accel.c, timestep.c)
  asmth, rcut, G, softening, mass, boxsize, timebase_interval: the constants
and, in ref_n16_pm32_mixed.npz, eight passes of the run loop on a box whose
particles take different individual timesteps (see mixed() below); and, in
ref_n32_pm64.npz, the forces of the small workload's box (32^3 particles,
L = 100 Mpc/h, PMGRID = 64, softening 0.03 of the mean spacing) on a seeded
subsample of 4096 targets (see small_workload() below).
The keys/permutation fixture uses the oracle's restatement of calcHashD plus
a stable sort (the reference computes keys only on the GPU, which does not
build on CUDA 13); it is pinned by tests/test_oracle_ref.py.

Usage: python tests/golden/make_golden.py [n16] [n32]   (default: both)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from cuco_gb300 import ics  # noqa: E402

N_SIDE, BOX_MPC, Z, SEED, PMGRID = 16, 50.0, 49.0, 2024, 32
FACTOR_PAIRS = [(0, 1 << 20), (1 << 20, 1 << 22), (5, 1 << 27), (1 << 27, 1 << 28)]


def main():
    ic = ics.zeldovich(N_SIDE, BOX_MPC, Z, SEED)
    eps = float(np.float32(0.03 * ic.boxsize / N_SIDE))
    ref = oracle.Reference(PMGRID)
    ref.begrun(ic, a_max=1.0, soft_comoving=eps, max_dloga=0.03, errtol=0.025)
    pos, vel, _, _ = ref.get()
    acc_pp = ref.pp(1)
    acc_pm = ref.pm()
    drift, kick = ref.tables()
    factors = np.array([[ref.lib.cref_drift_factor(a, b), ref.lib.cref_kick_factor(a, b)]
                        for a, b in FACTOR_PAIRS])
    out = dict(pos=pos, vel=vel, acc_pp=acc_pp, acc_pm=acc_pm, drift=drift, kick=kick,
               factor_pairs=np.array(FACTOR_PAIRS), factors=factors, asmth=ref.asmth, rcut=ref.rcut,
               G=ref.G, softening=ref.softening, mass=ic.mass, boxsize=ic.boxsize,
               timebase_interval=ref.timebase_interval, a_begin=np.float32(ic.a), pmgrid=PMGRID,
               eps=eps)
    port = oracle.Port()
    G = PMGRID
    gf = np.float32(np.float32(G) / np.float32(ic.boxsize))
    keys = port.keys(pos, gf, G)
    sk, perm = port.stable_sort(keys, G ** 3)
    out.update(keys=keys, sorted_keys=sk, perm=perm)
    # three passes of the reference run loop (fresh begrun: the loop starts at Ti = 0)
    ref2 = oracle.Reference(PMGRID)
    ref2.begrun(ic, a_max=1.0, soft_comoving=eps, max_dloga=0.03, errtol=0.025)
    ti = []
    for _ in range(3):
        ti.append(ref2.step(1))
    rp, rv, rpp, rpm = ref2.get()
    b, e, pm = ref2.timeline()
    out.update(run_pos=rp, run_vel=rv, run_acc_pp=rpp, run_acc_pm=rpm, run_ti_beg=b, run_ti_end=e,
               run_pm_ti=pm, run_ti_current=np.array(ti))
    np.savez_compressed(os.path.join(HERE, "ref_n16_pm32.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_n16_pm32.npz"), "Ti:", ti, "steps:", np.unique(e - b))
    mixed()


# A box clustered enough (z = 4) and a tolerance tight enough (ErrTolIntAccuracy
# = 0.005) that the particles take three different power-of-two steps below the
# PM step: eight passes of the run loop exercise the individual timesteps
# (timestep.c:11-94) - which particles are kicked, when the PM kick comes, and
# the drift of inactive particles between their kicks.
MIXED_Z, MIXED_ERRTOL, MIXED_SEED, MIXED_PASSES = 4.0, 0.005, 7, 8


def mixed():
    ic = ics.zeldovich(N_SIDE, BOX_MPC, MIXED_Z, MIXED_SEED)
    eps = float(np.float32(0.03 * ic.boxsize / N_SIDE))
    ref = oracle.Reference(PMGRID)
    ref.begrun(ic, a_max=1.0, soft_comoving=eps, max_dloga=0.03, errtol=MIXED_ERRTOL)
    pos0, vel0, _, _ = ref.get()
    ti = [ref.step(1) for _ in range(MIXED_PASSES)]
    rp, rv, rpp, rpm = ref.get()
    b, e, pm = ref.timeline()
    out = dict(pos=pos0, vel=vel0, mass=ic.mass, boxsize=ic.boxsize, a_begin=np.float32(ic.a), pmgrid=PMGRID,
               eps=eps, errtol=MIXED_ERRTOL, max_dloga=0.03, run_pos=rp, run_vel=rv, run_acc_pp=rpp,
               run_acc_pm=rpm, run_ti_beg=b, run_ti_end=e, run_pm_ti=pm, run_ti_current=np.array(ti))
    path = os.path.join(HERE, "ref_n16_pm32_mixed.npz")
    np.savez_compressed(path, **out)
    steps, counts = np.unique(e - b, return_counts=True)
    print("wrote", path, "Ti:", ti, "steps:", dict(zip(steps.tolist(), counts.tolist())))


SMALL_N_SIDE, SMALL_BOX_MPC, SMALL_SEED, SMALL_PMGRID, SMALL_TARGETS = 32, 100.0, 1, 64, 4096


def small_workload():
    """The small workload's box at z = 49: all positions, and the reference's
    short-range and PM forces on a seeded subsample of targets."""
    ic = ics.zeldovich(SMALL_N_SIDE, SMALL_BOX_MPC, Z, SMALL_SEED)
    eps = float(np.float32(0.03 * ic.boxsize / SMALL_N_SIDE))
    ref = oracle.Reference(SMALL_PMGRID)
    ref.begrun(ic, soft_comoving=eps)
    pos = ref.get()[0]
    acc_pp = ref.pp(8)
    acc_pm = ref.pm()
    sub = np.sort(np.random.default_rng(SMALL_TARGETS).choice(ic.n, SMALL_TARGETS, replace=False))
    out = dict(pos=pos, targets=sub, acc_pp=acc_pp[sub], acc_pm=acc_pm[sub], asmth=ref.asmth, rcut=ref.rcut,
               G=ref.G, softening=ref.softening, mass=ic.mass, boxsize=ic.boxsize, pmgrid=SMALL_PMGRID, eps=eps)
    path = os.path.join(HERE, "ref_n32_pm64.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    which = sys.argv[1:] or ["n16", "n32"]
    if "n16" in which:
        main()
    if "n32" in which:
        small_workload()
