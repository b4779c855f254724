"""The oracle against the golden fixtures made by the reference itself
(tests/golden/make_golden.py).  These run anywhere, including hosts without
the reference sources, so they pin the oracle wherever the GPU tests use it."""
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "ref_n16_pm32.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(FIX))


def params(g):
    return oracle.OpParams(float(g["boxsize"]), float(np.float32(g["mass"])), float(g["G"]),
                           float(g["asmth"]), float(g["rcut"]), float(g["softening"]))


def test_golden_pp_pm_bit_exact(port, gold):
    p = params(gold)
    M = int(gold["pmgrid"])
    assert np.array_equal(port.pp(gold["pos"], p, M, 4), gold["acc_pp"])
    assert np.array_equal(port.pm(gold["pos"], p, M, 4), gold["acc_pm"])


def test_golden_tables_and_factors(port, gold):
    a0 = float(gold["a_begin"])
    d64, k64 = port.drift_tables(a0, 1.0, 0.3, 0.7, 0.1)
    assert np.max(np.abs(d64.astype(np.float32).view(np.int32) - gold["drift"].view(np.int32))) <= 1
    assert np.max(np.abs(k64.astype(np.float32).view(np.int32) - gold["kick"].view(np.int32))) <= 1
    tbi = float(gold["timebase_interval"])
    for (t0, t1), (fd, fk) in zip(gold["factor_pairs"], gold["factors"]):
        assert port.table_factor(gold["drift"].astype(np.float64), np.log(a0), 0.0, tbi, int(t0), int(t1)) == fd
        assert port.table_factor(gold["kick"].astype(np.float64), np.log(a0), 0.0, tbi, int(t0), int(t1)) == fk


def test_golden_keys_and_permutation(port, gold):
    G = int(gold["pmgrid"])
    gf = np.float32(np.float32(G) / np.float32(gold["boxsize"]))
    keys = port.keys(gold["pos"], gf, G)
    assert np.array_equal(keys, gold["keys"])
    sk, perm = port.stable_sort(keys, G ** 3)
    assert np.array_equal(perm, gold["perm"])
    assert np.array_equal(sk, gold["sorted_keys"])


def test_golden_small_workload_bit_exact(port):
    """The small workload's box (32^3, PMGRID 64): the restatement's short range
    and PM on the fixture's targets equal the reference's, bit for bit."""
    g = dict(np.load(os.path.join(HERE, "golden", "ref_n32_pm64.npz")))
    p = params(g)
    M, tg = int(g["pmgrid"]), g["targets"]
    assert np.array_equal(port.pp_targets(g["pos"], tg, p, M, 4), g["acc_pp"])
    assert np.array_equal(port.pm(g["pos"], p, M, 4)[tg], g["acc_pm"])
