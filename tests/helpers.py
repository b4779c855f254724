"""Shared inputs for the parity tests (seeded, small enough for the CPU oracle)."""
import numpy as np

from cuco_gb300 import ics


def zeldovich(n_side=32, box_mpc=100.0, z=49.0, seed=1):
    return ics.zeldovich(n_side, box_mpc, z, seed)


def softening_h(boxsize, n_side, frac=0.03):
    """Spline length h = 2.8 eps with eps = frac * mean spacing (gravlist.cpp:36)."""
    return float(np.float32(2.8 * np.float32(frac * boxsize / n_side)))


def clustered(n, boxsize, seed, nblobs=3, frac_in_blobs=0.6, radius=0.004):
    """Uniform background plus tight Gaussian blobs: cells with thousands of
    particles, to drive the chunked short-range paths."""
    rng = np.random.default_rng(seed)
    nb = int(n * frac_in_blobs)
    pos = rng.uniform(0, boxsize, size=(n, 3))
    centres = rng.uniform(0, boxsize, size=(nblobs, 3))
    which = rng.integers(0, nblobs, size=nb)
    pos[:nb] = centres[which] + rng.normal(0, radius * boxsize, size=(nb, 3))
    pos = np.mod(pos, boxsize).astype(np.float32)
    pos[pos >= np.float32(boxsize)] = 0
    return pos
