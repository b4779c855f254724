"""The debug build's bounds checks, in place of a memory checker: the library
compiled with CUCO_BOUNDS_CHECK (libcuco_gb300_debug.so) runs small uniform
and clustered boxes, both forms, dense cells staged in chunks, a few steps and
an ensemble of mixed meshes, and no kernel index may leave its bounds.  Runs
in a child process that loads the debug build in place of the release one."""
import os
import subprocess
import sys

import pytest

from cuco_gb300 import _native, build

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import ctypes, sys
sys.path.insert(0, %(root)r)
sys.path.insert(0, %(tests)r)
import numpy as np
from cuco_gb300 import Box, BoxConfig, ics, fixed_step_schedule, _native
from cuco_gb300.engine import MODE_FIXED
from cuco_gb300.ensemble import Ensemble
from helpers import clustered
lib = _native.load()
assert lib._name.endswith("_debug.so"), lib._name
for mode in (0, MODE_FIXED):
    ic = ics.zeldovich(32, 100.0, 49.0, 2)
    soft = 2.8 * 0.03 * ic.boxsize / 32
    box = Box(BoxConfig(n=ic.n, pm_grid=64, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                        softening=soft, mode=mode))
    box.set_state(ic.pos, ic.canonical_velocity())
    _, drift, kick = fixed_step_schedule(ic.a, 1.0, 20)
    for s in range(4):
        box.step(drift[s], kick[s])
    box.close()
    pos = clustered(20000, ic.boxsize, seed=3, nblobs=2, frac_in_blobs=0.8, radius=0.002)
    box = Box(BoxConfig(n=pos.shape[0], pm_grid=64, cell_grid=16, boxsize=ic.boxsize, mass=ic.mass,
                        G=ics.G_INTERNAL, softening=soft, mode=mode))
    box.set_state(pos)
    box.forces()
    box.close()
cfgs, ics_ = [], []
for k, (n, L) in enumerate([(16, 60.0), (20, 80.0), (24, 90.0)]):
    ic = ics.zeldovich(n, L, 49.0, 10 + k)
    ics_.append(ic)
    cfgs.append(BoxConfig(n=ic.n, pm_grid=2 * n, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                          softening=2.8 * 0.025 * ic.boxsize / n, mode=MODE_FIXED))
ens = Ensemble(cfgs)
for b, ic in enumerate(ics_):
    ens.set_state(b, ic.pos, ic.canonical_velocity())
ens.forces()
ens.step(np.full(3, 1e-3), np.full(3, 1e-3))
ens.sync()
ens.close()
count = ctypes.c_uint64()
assert lib.cuco_debug_bounds_violations(ctypes.byref(count)) == 0, lib.cuco_last_error()
print("violations", count.value)
"""


def test_debug_build_finds_no_out_of_bounds_index():
    lib_path = build.build(debug=True)
    env = dict(os.environ, CUCO_LIBRARY=lib_path)
    code = SCRIPT % {"root": ROOT, "tests": os.path.join(ROOT, "tests")}
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "violations 0" in r.stdout, r.stdout[-2000:]


def test_release_build_has_no_bounds_checks():
    import ctypes
    lib = _native.load()
    assert lib.cuco_debug_bounds_violations(ctypes.byref(ctypes.c_uint64())) == 6  # CUCO_ERR_UNSUPPORTED
