"""The reference-named entry points, driven exactly as the reference's host code
drives them (gravlist.cpp:48-193, pm_periodic.c, driftfac.c), against the CPU
oracle.  Device buffers come from the library's own allocateArray."""
import ctypes

import numpy as np
import pytest

import oracle
from cuco_gb300 import _native, ics
from cuco_gb300._native import All, Header, Particle, SimParam, SoftParam
from helpers import softening_h, zeldovich
from conftest import rms_rel

pytestmark = pytest.mark.gpu


def dev_alloc(lib, nbytes):
    p = ctypes.c_void_p()
    lib.allocateArray(ctypes.byref(p), nbytes)
    return p


def to_dev(lib, arr):
    arr = np.ascontiguousarray(arr)
    d = dev_alloc(lib, arr.nbytes)
    lib.copyArrayToDevice(d, arr.ctypes.data, 0, arr.nbytes)
    return d


def from_dev(lib, d, shape, dtype):
    out = np.empty(shape, dtype=dtype)
    lib.copyArrayFromDevice(out.ctypes.data, d, out.nbytes)
    return out


def simparam(boxsize, G, mass, asmth, rcut):
    sp = SimParam()
    tab = oracle.Port().shortrange_table()
    for i in range(1000):
        sp.shortrange_table[i] = tab[i]
    sp.boxsize = boxsize
    sp.boxhalf = boxsize / 2
    sp.to_grid_fac = np.float32(np.float32(G) / np.float32(boxsize))
    sp.rcut = rcut
    sp.rcut2 = float(np.float32(np.float64(rcut) * rcut))
    sp.asmth = asmth
    sp.asmthfac = float(np.float32(0.5 / np.float64(asmth) * (1000 / 3.0)))
    sp.mass = mass
    sp.G = ics.G_INTERNAL
    return sp


def test_gravlist_gpu_pipeline_matches_oracle(port):
    """calcHash -> radixSort -> reorderDataAndFindCellStart ->
    cudaForceEvaluateShortrange, with the reference's buffer shapes."""
    lib = _native.load()
    lib.cudaInit()
    ic = zeldovich(32, 100.0)
    n, G = ic.n, 64
    lib.cuco_dropin_configure(64, G)
    p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, 64, softening_h(ic.boxsize, 32))
    lib.setSimParam(ctypes.byref(simparam(ic.boxsize, G, ic.mass, p.asmth, p.rcut)))
    soft = SoftParam(p.softening, 1.0 / p.softening, (1.0 / p.softening) ** 3)
    lib.setSoftParam(ctypes.byref(soft))
    pos4 = np.zeros((n, 4), dtype=np.float32)
    pos4[:, :3] = ic.pos
    d_pos = to_dev(lib, pos4)
    d_hash, d_idx = dev_alloc(lib, 4 * n), dev_alloc(lib, 4 * n)
    lib.calcHash(d_hash, d_idx, d_pos, n)
    # RadixSort temporaries as radixsort.h:252-276 sizes them
    nb = (n + 1023) // 1024
    d_tk, d_tv = dev_alloc(lib, 4 * n), dev_alloc(lib, 4 * n)
    d_c, d_cs, d_bo = (dev_alloc(lib, 4 * 32 * nb) for _ in range(3))
    lib.radixSort(d_hash, d_idx, d_tk, d_tv, d_c, d_cs, d_bo, 0, n, 18, False)
    keys = from_dev(lib, d_hash, n, np.uint32)
    perm = from_dev(lib, d_idx, n, np.uint32)
    k_ref = port.keys(ic.pos, np.float32(np.float32(G) / np.float32(ic.boxsize)), G)
    sk_ref, perm_ref = port.stable_sort(k_ref, G ** 3)
    assert np.array_equal(keys, sk_ref)
    assert np.array_equal(perm, perm_ref)
    ncell = G ** 3
    d_start, d_end, d_spos = dev_alloc(lib, 4 * ncell), dev_alloc(lib, 4 * ncell), dev_alloc(lib, 16 * n)
    lib.reorderDataAndFindCellStart(d_start, d_end, d_spos, d_hash, d_idx, d_pos, n, ncell)
    cs = from_dev(lib, d_start, ncell, np.uint32)
    ce = from_dev(lib, d_end, ncell, np.uint32)
    cs_ref, ce_ref = port.cell_bounds(sk_ref, ncell)
    assert np.array_equal(cs, cs_ref)
    ne = cs_ref != 0xFFFFFFFF
    assert np.array_equal(ce[ne], ce_ref[ne])
    spos = from_dev(lib, d_spos, (n, 4), np.float32)
    assert np.array_equal(spos[:, :3], ic.pos[perm_ref])
    d_acc = dev_alloc(lib, 16 * n)
    lib.cudaForceEvaluateShortrange(d_acc, d_spos, d_idx, d_start, d_end, n, ncell)
    acc = from_dev(lib, d_acc, (n, 4), np.float32)
    ref = port.pp(ic.pos, p, G, 8)
    assert rms_rel(acc[:, :3], ref) < 1e-4
    assert np.all(acc[:, 3] == 0)
    lib.checkCudaError(b"gravlist pipeline")
    for d in (d_pos, d_hash, d_idx, d_tk, d_tv, d_c, d_cs, d_bo, d_start, d_end, d_spos, d_acc):
        lib.freeArray(d)


def test_radixsort_keys_only_and_small(port):
    lib = _native.load()
    for n, bits in [(1, 18), (33, 18), (1025, 24), (70000, 18), (70000, 12)]:
        rng = np.random.default_rng(n + bits)
        k = rng.integers(0, 1 << bits, size=n, dtype=np.uint32)
        d_k = to_dev(lib, k)
        nb = (n + 1023) // 1024
        d_t = dev_alloc(lib, 4 * n)
        d_c, d_cs, d_bo = (dev_alloc(lib, 4 * 32 * nb) for _ in range(3))
        lib.radixSortKeysOnly(d_k, d_t, d_c, d_cs, d_bo, 0, n, bits, False)
        assert np.array_equal(from_dev(lib, d_k, n, np.uint32), np.sort(k))
        for d in (d_k, d_t, d_c, d_cs, d_bo):
            lib.freeArray(d)


class DropIn:
    """The reference's globals inside libcuco_gb300.so, set as begrun() would."""

    def __init__(self, ic, pmgrid, cellgrid, soft_eps, a_max=1.0):
        lib = self.lib = _native.load()
        self.n = ic.n
        self.parts = (Particle * ic.n)()
        arr = np.ctypeslib.as_array(self.parts)
        raw = arr.view(np.uint8).reshape(ic.n, 60).view(np.float32)
        raw[:, 0:3] = ic.pos
        raw[:, 3] = ic.mass
        raw[:, 4:7] = ic.canonical_velocity()
        ctypes.c_void_p.in_dll(lib, "P").value = ctypes.addressof(self.parts)
        ctypes.c_uint.in_dll(lib, "NumPart").value = ic.n
        hdr = Header.in_dll(lib, "header")
        hdr.NumPart, hdr.Mass, hdr.Time, hdr.BoxSize = ic.n, ic.mass, ic.a, ic.boxsize
        al = self.All = All.in_dll(lib, "All")
        al.NumPart, al.BoxSize, al.Mass = ic.n, ic.boxsize, ic.mass
        al.G, al.Hubble = ics.G_INTERNAL, ics.HUBBLE_INTERNAL
        al.Omega0, al.OmegaLambda, al.HubbleParam = 0.3, 0.7, 0.7
        al.Time = al.TimeBegin = ic.a
        al.TimeMax = a_max
        al.Timebase_interval = (np.log(a_max) - np.log(np.float32(ic.a))) / (1 << 28)
        al.Ti_Current = 0
        al.SofteningHalo, al.SofteningHaloMaxPhys = soft_eps, 1e30
        al.ErrTolIntAccuracy, al.MaxSizeTimestep = 0.025, 0.03
        lib.cuco_dropin_configure(pmgrid, cellgrid)
        lib.set_softenings()
        lib.long_range_init()
        lib.linklist_init()
        lib.init_drift_table()

    def field(self, name):
        arr = np.ctypeslib.as_array(self.parts).view(np.uint8).reshape(self.n, 60).view(np.float32)
        sl = {"Pos": slice(0, 3), "Vel": slice(4, 7), "GravAccel": slice(7, 10), "GravPM": slice(10, 13)}[name]
        return arr[:, sl].copy()


def test_dropin_forces_match_oracle(port):
    ic = zeldovich(32, 100.0, seed=4)
    eps = np.float32(0.03 * ic.boxsize / 32)
    d = DropIn(ic, 64, 64, eps)
    lib = d.lib
    assert abs(d.All.Asmth - np.float32(1.25 * ic.boxsize / 64)) == 0
    lib.gravity_linklist_cuda()
    lib.pmforce_periodic()
    p = oracle.reference_params(ic.boxsize, ic.mass, ics.G_INTERNAL, 64, d.All.ForceSoftening)
    assert rms_rel(d.field("GravAccel"), port.pp(ic.pos, p, 64, 8)) < 1e-4
    assert rms_rel(d.field("GravPM"), port.pm(ic.pos, p, 64, 8)) < 1e-4
    assert np.array_equal(d.field("Pos"), ic.pos)


def test_dropin_drift_factors_and_move(port):
    ic = zeldovich(16, 50.0, seed=2)
    d = DropIn(ic, 32, 32, np.float32(0.03 * ic.boxsize / 16))
    lib = d.lib
    # drift_integ reads All.Omega0, All.OmegaLambda, All.Hubble: floats (allvars.h:73-75)
    f32 = lambda v: float(np.float32(v))  # noqa: E731
    drift, kick = port.drift_tables(f32(ic.a), 1.0, f32(0.3), f32(0.7), f32(ics.HUBBLE_INTERNAL))
    l0, l1, tbi = np.log(float(np.float32(ic.a))), np.log(1.0), d.All.Timebase_interval
    for t0, t1 in [(0, 1 << 20), (1 << 20, 1 << 24), (12345, 1 << 28)]:
        assert lib.get_drift_factor(t0, t1) == pytest.approx(port.table_factor(drift, l0, l1, tbi, t0, t1), rel=1e-12)
        assert lib.get_gravkick_factor(t0, t1) == pytest.approx(port.table_factor(kick, l0, l1, tbi, t0, t1), rel=1e-12)
    vel = d.field("Vel").astype(np.float64)
    pos0 = d.field("Pos").astype(np.float64)
    lib.move_particles(0, 1 << 22)
    dt = lib.get_drift_factor(0, 1 << 22)
    expect = (pos0 + vel * dt).astype(np.float32)
    assert np.array_equal(d.field("Pos"), expect)
