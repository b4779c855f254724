"""A C++ host that keeps the reference's gravlist.cpp way of sorting - its
own `sorter = new RadixSort(numParticles)` and `sorter->sort(hash, index, n,
18)` (gravlist.cpp:98,164-167) - compiled with g++ against include/radixsort.h
and include/cuco_gb300.h only, linked with libcuco_gb300.so.  Its keys,
permutation, cell bounds and sorted positions must equal the oracle's bit for
bit; the keys-only and float-key overloads of RadixSort::sort must equal
numpy's stable sorts."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from cuco_gb300 import _native
from helpers import zeldovich

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def host_exe(tmp_path_factory):
    _native.load()  # builds the library if needed
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("host") / "gravlist_host")
    lib_dir = os.path.dirname(_native.LIB_PATH)
    cmd = [gxx, "-O1", "-std=c++11", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "gravlist_host.cpp"), "-L", lib_dir, "-lcuco_gb300",
           "-Wl,-rpath," + lib_dir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("n_side,G", [(32, 64), (20, 32)])
def test_reference_style_host_sort_pipeline(port, host_exe, tmp_path, n_side, G):
    ic = zeldovich(n_side, 100.0, seed=3)
    n, L = ic.n, np.float32(ic.boxsize)
    rng = np.random.default_rng(n)
    fkeys = rng.normal(0, 100, n).astype(np.float32)
    fkeys[: n // 4] = fkeys[0]  # runs of equal keys: stability
    src, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(src, "wb") as f:
        np.array([n, G], dtype=np.int32).tofile(f)
        np.array([L], dtype=np.float32).tofile(f)
        ic.pos.astype(np.float32).tofile(f)
        fkeys.tofile(f)
    r = subprocess.run([host_exe, str(src), str(out)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(out, dtype=np.uint32)
    nc = G ** 3
    parts = np.split(raw, np.cumsum([n, n, nc, nc, 4 * n, n, n]))
    hash_, index, start, end, sorted4, keys_only, fsorted, fvals = parts
    k_ref = port.keys(ic.pos, np.float32(np.float32(G) / L), G)
    sk_ref, perm_ref = port.stable_sort(k_ref, nc)
    st_ref, en_ref = port.cell_bounds(sk_ref, nc)
    assert np.array_equal(hash_, sk_ref)
    assert np.array_equal(index, perm_ref)
    assert np.array_equal(start, st_ref)
    occupied = st_ref != 0xFFFFFFFF
    assert np.array_equal(end[occupied], en_ref[occupied])
    sp = sorted4.view(np.float32).reshape(n, 4)[:, :3]
    assert np.array_equal(sp, ic.pos[perm_ref])
    assert np.array_equal(keys_only, sk_ref)
    order = np.argsort(fkeys, kind="stable")
    assert np.array_equal(fsorted.view(np.float32), fkeys[order])
    assert np.array_equal(fvals, order.astype(np.uint32))
