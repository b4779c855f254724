"""Several boxes in one process, as a serving loop holds them: boxes of
different mixed-radix meshes, created one after the other, each keep working
(the transforms' shared-memory limit is a per-kernel attribute that a later
box must not lower under an earlier one's launches)."""
import numpy as np
import pytest

import oracle
from cuco_gb300 import Box, BoxConfig, ics
from conftest import rms_rel

pytestmark = pytest.mark.gpu


def _box(n_side, L, seed):
    ic = ics.zeldovich(n_side, L, 49.0, seed)
    M = 2 * n_side
    soft = float(np.float32(2.8 * np.float32(0.025 * ic.boxsize / n_side)))
    box = Box(BoxConfig(n=ic.n, pm_grid=M, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL, softening=soft))
    box.set_state(ic.pos, ic.canonical_velocity())
    return ic, M, soft, box


def test_boxes_of_different_meshes(port):
    big = _box(96, 300.0, 5)    # M = 192: its z passes need more than 48 KB of shared memory
    small = _box(20, 60.0, 6)   # M = 40, created after it
    for ic, M, soft, box in (big, small):
        box.forces()
        _, _, app, apm = box.get_state()
        p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, M, soft)
        err = rms_rel(apm, port.pm(ic.pos, p, M, 16))
        print(f"M={M}: pm {err:.2e}")
        assert np.isfinite(app).all() and err < 1e-4
    for _, _, _, box in (big, small):
        box.close()
