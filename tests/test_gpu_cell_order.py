"""The short range's source order: the sort's cells, each refined by z slice.

Within every cell the particles are grouped into 8 slices of the cell along z,
in increasing slice order and stable within a slice (the sort's order).  The
slice is taken from the key rule's float product (G/L) * z for float positions
and from the three bits below the cell index of z * G / 2^32 for fixed point.
The order and the slices are compared bit for bit with numpy, for cells of a
few particles (one warp pass) and for dense cells of thousands (chunked).
"""
import numpy as np
import pytest

from cuco_gb300 import Box, BoxConfig, ics
from cuco_gb300.engine import MODE_FIXED
from helpers import clustered, softening_h, zeldovich

pytestmark = pytest.mark.gpu


def expected(keys, perm, G, slice_of_original):
    sl = slice_of_original[perm]
    # cells ascending (keys are sorted), then slice, then the sort's order
    order = np.lexsort((np.arange(keys.size), sl, keys))
    return perm[order], sl[order].astype(np.float32)


def plain_slices(pos, keys_orig, G, L):
    gridfac = np.float32(G) / np.float32(L)
    t = pos[:, 2].astype(np.float32) * gridfac
    cz = (keys_orig % G).astype(np.float32)
    s = np.floor((t - cz) * np.float32(8)).astype(np.int64)
    return np.clip(s, 0, 7)


@pytest.mark.parametrize("kind", ["zeldovich", "clustered", "ragged"])
def test_cell_order_plain(kind):
    if kind == "zeldovich":
        ic = zeldovich(32, 100.0)
        pos, L, G = ic.pos, ic.boxsize, 16
    elif kind == "clustered":
        L, G = 100000.0, 16
        pos = clustered(30000, L, seed=3)
    else:
        L, G = 500.0, 8
        pos = np.random.default_rng(4).uniform(0, L, size=(1001, 3)).astype(np.float32)
    n = pos.shape[0]
    box = Box(BoxConfig(n=n, pm_grid=2 * G, cell_grid=G, boxsize=L, mass=1.0, G=ics.G_INTERNAL,
                        softening=softening_h(L, 32)))
    box.set_state(pos)
    box.forces(pm=False, pp=True)
    keys, perm, _, _ = box.debug()
    perm_s, sl = box.cell_order()
    held = box.get_state()[0]
    keys_orig = np.empty(n, dtype=np.uint32)
    keys_orig[perm] = keys
    want_perm, want_sl = expected(keys, perm, G, plain_slices(held, keys_orig, G, L))
    assert np.array_equal(perm_s, want_perm)
    assert np.array_equal(sl, want_sl)
    if kind == "clustered":
        assert np.bincount(keys).max() > 32  # the chunked path ran
    box.close()


def test_cell_order_fixed():
    L, G = 100000.0, 16
    pos = clustered(30000, L, seed=6)
    n = pos.shape[0]
    box = Box(BoxConfig(n=n, pm_grid=32, cell_grid=G, boxsize=L, mass=1.0, G=ics.G_INTERNAL,
                        softening=softening_h(L, 32), mode=MODE_FIXED))
    box.set_state(pos)
    box.forces(pm=False, pp=True)
    keys, perm, _, _ = box.debug()
    perm_s, sl = box.cell_order()
    u = box.get_state_fixed()
    s = ((u[:, 2].astype(np.uint64) * np.uint64(G)) >> np.uint64(29)) & np.uint64(7)
    want_perm, want_sl = expected(keys, perm, G, s.astype(np.int64))
    assert np.array_equal(perm_s, want_perm)
    assert np.array_equal(sl, want_sl)
    box.close()
