"""The largest mesh (M = 1024, the 32x32 register transform) against the oracle,
and the large box (512^3 particles, L = 1000 Mpc/h, M = 1024) in both forms
on a seeded 4096-particle subsample at z = 49.

The oracle's PM at M = 1024 works on a full double-precision complex grid
(~26 GB of host memory, about a minute on 16 cores); the 512^3 initial
conditions take about a minute to generate.  Bars as for the smaller meshes:
the plain form within 1e-4 rms of the reference's force path, the precision
form within 1e-3."""
import os

import numpy as np
import pytest

import oracle
from cuco_gb300 import Box, BoxConfig, ics
from cuco_gb300.engine import MODE_FIXED
from conftest import rms_rel
from helpers import clustered

pytestmark = pytest.mark.gpu

THREADS = min(32, os.cpu_count() or 1)


def test_pm_mesh_1024_vs_oracle(port):
    ic = ics.zeldovich(64, 1000.0, 49.0, seed=17)
    # plus dense blobs: power at every wave number of the mesh
    blobs = clustered(65536, ic.boxsize, seed=18, nblobs=4, frac_in_blobs=1.0, radius=0.002)
    pos = np.concatenate([ic.pos, blobs]).astype(np.float32)
    M = 1024
    soft = 2.8 * 0.025 * ic.boxsize / 512
    box = Box(BoxConfig(n=pos.shape[0], pm_grid=M, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                        softening=soft))
    box.set_state(pos)
    box.forces(pm=True, pp=False)
    apm = box.get_state()[3]
    box.close()
    p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, M, soft)
    ref = port.pm(pos, p, M, THREADS)
    err = rms_rel(apm, ref)
    print(f"PM M=1024: rms {err:.2e}")
    assert err < 1e-4


def rounded_to_fixed(pos, L):
    u = (np.rint(pos.astype(np.float64) * (2.0 ** 32 / L)).astype(np.int64) & 0xFFFFFFFF)
    return (u.astype(np.float64) * (L / 2.0 ** 32)).astype(np.float32)


def test_large_box_both_forms_vs_reference_path(port):
    N, L, M = 512, 1000.0, 1024
    ic = ics.zeldovich(N, L, 49.0, seed=12345)
    soft = float(np.float32(2.8 * np.float32(0.025 * ic.boxsize / N)))
    sub = np.sort(np.random.default_rng(4096).choice(ic.n, 4096, replace=False))
    p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, M, soft)
    errs = {}
    for mode, name in ((0, "plain"), (MODE_FIXED, "precision")):
        box = Box(BoxConfig(n=ic.n, pm_grid=M, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                            softening=soft, mode=mode))
        box.set_state(ic.pos)
        box.forces()
        _, _, app, apm = box.get_state()
        box.close()
        app, apm = app[sub].copy(), apm[sub].copy()
        pref = rounded_to_fixed(ic.pos, ic.boxsize) if mode else ic.pos
        # the oracle's cell grid only orders its sums: any grid whose cells
        # cover the cut gives the same pairs; 256^3 keeps its lists small
        ref_pp = port.pp_targets(pref, sub, p, 256, THREADS)
        ref_pm = port.pm(pref, p, M, THREADS)[sub]
        errs[name] = (rms_rel(app, ref_pp), rms_rel(apm, ref_pm), rms_rel(app + apm, ref_pp + ref_pm))
        del pref
    for name, (e_pp, e_pm, e_tot) in errs.items():
        print(f"512^3 M=1024 z=49 {name:9s}: pp {e_pp:.2e}  pm {e_pm:.2e}  total {e_tot:.2e}")
    assert max(errs["plain"]) < 1e-4
    assert max(errs["precision"]) < 1e-3
