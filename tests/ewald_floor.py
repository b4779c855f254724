"""The reference method's force error against the FP64 Ewald sum (the method
floor) on a box too large for the GPU test suite's time: the oracle's
restatement of the reference's force path (bit-exact with it) against the
oracle's Ewald sum, on a seeded subsample of targets, at the initial
conditions.  Prints the rms relative error and the median and 99th
percentile of the per-particle relative error, for the short range plus PM.

    python tests/ewald_floor.py --n-side 512 --box 1000 --mesh 1024

The 512^3 box (L = 1000 Mpc/h, M = 1024, softening 0.025 of the mean spacing,
seed 12345, 4096 targets) is the large-box workload's and matches
test_gpu_large_mesh.py's state and subsample; it needs ~40 GB of host memory
and about an hour on 8 cores, most of it the Ewald sum over 1.3e8 sources.
"""
import argparse
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import oracle  # noqa: E402
from conftest import err_stats  # noqa: E402
from cuco_gb300 import ics  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-side", type=int, default=512)
    ap.add_argument("--box", type=float, default=1000.0, help="Mpc/h")
    ap.add_argument("--mesh", type=int, default=1024)
    ap.add_argument("--seed", type=int, default=12345)
    ap.add_argument("--targets", type=int, default=4096)
    ap.add_argument("--cell-grid", type=int, default=256, help="the oracle's cell grid for the short range")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()

    t0 = time.time()
    ic = ics.zeldovich(a.n_side, a.box, 49.0, seed=a.seed)
    soft = float(np.float32(2.8 * np.float32(0.025 * ic.boxsize / a.n_side)))
    sub = np.sort(np.random.default_rng(a.targets).choice(ic.n, a.targets, replace=False))
    p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, a.mesh, soft)
    port = oracle.Port()
    print(f"initial conditions {time.time() - t0:.0f} s", flush=True)

    t = time.time()
    acc = port.pp_targets(ic.pos, sub, p, a.cell_grid, a.threads).astype(np.float64)
    acc += port.pm(ic.pos, p, a.mesh, a.threads)[sub]
    print(f"reference method (short range + PM) {time.time() - t:.0f} s", flush=True)

    t = time.time()
    L, mass = float(np.float32(ic.boxsize)), float(np.float32(ic.mass))
    tg = ic.pos[sub].astype(np.float64)
    src = ic.pos.astype(np.float64)
    del ic
    ew = port.ewald(src, mass, ics.G_INTERNAL, L, soft, tg, a.threads)
    print(f"Ewald {time.time() - t:.0f} s", flush=True)

    s = err_stats(acc, ew)
    print(f"FLOOR {a.n_side}^3 L={a.box:g} M={a.mesh} z=49, {a.targets} targets: "
          f"rms {s['rms']:.3e} median {s['median']:.3e} p99 {s['p99']:.3e}", flush=True)


if __name__ == "__main__":
    main()
