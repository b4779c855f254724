"""cuco_radix_sort_noalloc, the sort entry point that allocates no device
memory, against the allocating radixSort entry point.

The allocation-free sort is for callers that cannot call cudaMalloc where they
sort (it can synchronize the device and stall other streams; some hosts give
each job a fixed HBM slice up front).  Its scratch is one array built into the
library and shared by every call, so this checks two calls in a row: the
second must not see anything the first left behind.  Sorting is integer work:
the results must be identical.  This file is collected last so that a run
stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from cuco_gb300 import _native

pytestmark = pytest.mark.gpu


def _dev(lib, arr):
    arr = np.ascontiguousarray(arr, dtype=np.uint32)
    p = ctypes.c_void_p()
    lib.allocateArray(ctypes.byref(p), max(arr.nbytes, 4))
    if arr.nbytes:
        lib.copyArrayToDevice(p, arr.ctypes.data, 0, arr.nbytes)
    return p


def _host(lib, p, n):
    out = np.empty(n, dtype=np.uint32)
    if n:
        lib.copyArrayFromDevice(out.ctypes.data, p, out.nbytes)
    return out


def _sort_allocating(lib, keys, vals, bits):
    n = keys.size
    dk = _dev(lib, keys)
    dv = _dev(lib, vals) if vals is not None else None
    nb = (n + 1023) // 1024
    tmp = [ctypes.c_void_p() for _ in range(5)]
    for t, nbytes in zip(tmp, [4 * n, 4 * n, 128 * nb, 128 * nb, 128 * nb]):
        lib.allocateArray(ctypes.byref(t), max(nbytes, 4))
    if dv is None:
        lib.radixSortKeysOnly(dk, tmp[0], tmp[2], tmp[3], tmp[4], 0, n, bits, False)
    else:
        lib.radixSort(dk, dv, tmp[0], tmp[1], tmp[2], tmp[3], tmp[4], 0, n, bits, False)
    out = _host(lib, dk, n), (_host(lib, dv, n) if dv is not None else None)
    for p in [dk, *tmp] + ([dv] if dv is not None else []):
        lib.freeArray(p)
    return out


def _sort_noalloc(lib, keys, vals, bits):
    n = keys.size
    dk = _dev(lib, keys)
    dv = _dev(lib, vals) if vals is not None else None
    st = lib.cuco_radix_sort_noalloc(dk, dv, n, bits, None)
    assert st == 0, lib.cuco_last_error()
    lib.checkCudaError(b"cuco_radix_sort_noalloc")
    out = _host(lib, dk, n), (_host(lib, dv, n) if dv is not None else None)
    lib.freeArray(dk)
    if dv is not None:
        lib.freeArray(dv)
    return out


# (n, key bits, with values): the largest allowed n; an odd number of passes
# (result copied back from the scratch array); keys only; one tile (n <= 4096);
# an even number of passes (result already in place: 16 bits = two 8-bit
# passes, 32 bits = four); and n = 0
CASES = [(1 << 20, 18, True), (300001, 24, True), (300001, 24, False), (1000, 18, True), (1000, 18, False),
         (200000, 16, True), (70001, 32, True), (4096, 32, False), (0, 18, True)]


@pytest.mark.parametrize("n,bits,with_values", CASES)
def test_noalloc_sort_matches_allocating_sort_twice(n, bits, with_values):
    lib = _native.load()
    lib.cudaInit()
    for call in range(2):
        rng = np.random.default_rng(1000 * call + n + bits)
        keys = rng.integers(0, 1 << bits, size=n, dtype=np.uint64).astype(np.uint32)
        if call == 1:
            keys[: n // 3] = keys[0] if n else 0  # long runs of equal keys: stability
        vals = np.arange(n, dtype=np.uint32) if with_values else None
        k_ref, v_ref = _sort_allocating(lib, keys, vals, bits)
        k_na, v_na = _sort_noalloc(lib, keys, vals, bits)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(k_ref, keys[order])
        assert np.array_equal(k_na, k_ref)
        if with_values:
            assert np.array_equal(v_ref, order.astype(np.uint32))
            assert np.array_equal(v_na, v_ref)


def test_noalloc_rejects_more_than_the_fixed_limit():
    lib = _native.load()
    st = lib.cuco_radix_sort_noalloc(None, None, (1 << 20) + 1, 18, None)
    assert st == 1
    assert b"exceed" in lib.cuco_last_error()
