"""CPU oracle for the force path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package, and only as the checker or the timed CPU baseline.  The product
(cuco_gb300) never imports it.

Two CPU implementations are wrapped here:
  Port       - oracle/port.c + oracle/ewald.c, the project's C restatement of the
               reference algorithms (always buildable; runs on any host);
  Reference  - the reference's own CPU force path compiled from its sources by
               oracle/Makefile into oracle/_ref/ (only where the reference
               sources are present, i.e. not on a host without them).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")


def reference_dir() -> str:
    """Where the reference's sources lie: $CUCO_REFERENCE_DIR, else the
    location the oracle recipe (oracle/Makefile, REF) names."""
    env = os.environ.get("CUCO_REFERENCE_DIR")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build_port() -> str:
    r = subprocess.run(["make", "-s", "-C", HERE, "port"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle port build failed:\n" + r.stdout + r.stderr)
    return PORT_LIB


def reference_available() -> bool:
    d = reference_dir()
    return bool(d) and os.path.isfile(os.path.join(d, "gravlist.cpp"))


def build_reference(pmgrids=(32, 64, 128, 256)) -> list[str]:
    """Compile the reference's CPU path (one library per PM mesh size)."""
    if not reference_available():
        raise FileNotFoundError("reference sources not present at " + repr(reference_dir()))
    r = subprocess.run(["make", "-s", "-j4", "-C", HERE, "ref", "REF=" + reference_dir(),
                        "PMGRIDS=" + " ".join(str(m) for m in pmgrids)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference oracle build failed:\n" + r.stdout + r.stderr)
    return [os.path.join(REF_DIR, f"libcucoref_pm{m}.so") for m in pmgrids]


class OpParams(ctypes.Structure):
    _fields_ = [("boxsize", ctypes.c_float), ("mass", ctypes.c_float), ("G", ctypes.c_double),
                ("asmth", ctypes.c_float), ("rcut", ctypes.c_float),
                ("softening", ctypes.c_float)]


def reference_params(boxsize: float, mass: float, G: float, pmgrid: int, softening_h: float,
                     asmth_cells: float = 1.25, rcut_asmth: float = 4.5) -> OpParams:
    """Force parameters with the reference's float roundings
    (pm_periodic.c:27-28: Asmth and Rcut are stored as float)."""
    boxsize32 = np.float32(boxsize)
    asmth = np.float32(asmth_cells * float(boxsize32) / pmgrid)
    rcut = np.float32(rcut_asmth * float(asmth))
    return OpParams(float(boxsize32), float(np.float32(mass)), float(G), float(asmth), float(rcut),
                    float(np.float32(softening_h)))


class Port:
    """ctypes wrapper of oracle/_build/liboracle.so."""

    def __init__(self):
        if not os.path.isfile(PORT_LIB):
            build_port()
        lib = ctypes.CDLL(PORT_LIB)
        lib.op_keys.argtypes = [_f32p, ctypes.c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_int, _u32p]
        lib.op_stable_sort.argtypes = [_u32p, ctypes.c_int64, ctypes.c_uint32, _u32p, _u32p]
        lib.op_cell_bounds.argtypes = [_u32p, ctypes.c_int64, ctypes.c_uint32, _u32p, _u32p]
        lib.op_shortrange_table.argtypes = [_f32p]
        lib.op_pp.argtypes = [_f32p, ctypes.c_int64, ctypes.POINTER(OpParams), ctypes.c_int,
                              ctypes.c_int, _f32p]
        lib.op_pp_targets.argtypes = [_f32p, ctypes.c_int64,
                                      np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS"),
                                      ctypes.c_int64, ctypes.POINTER(OpParams), ctypes.c_int,
                                      ctypes.c_int, _f32p]
        lib.op_pair_count.argtypes = [_f32p, ctypes.c_int64, ctypes.POINTER(OpParams), ctypes.c_int,
                                      ctypes.c_int]
        lib.op_pair_count.restype = ctypes.c_int64
        lib.op_pm.argtypes = [_f32p, ctypes.c_int64, ctypes.POINTER(OpParams), ctypes.c_int,
                              ctypes.c_int, _f32p]
        lib.op_drift_tables.argtypes = [ctypes.c_double] * 5 + [ctypes.c_int, _f64p, _f64p]
        lib.op_table_factor.argtypes = [_f64p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int, ctypes.c_int]
        lib.op_table_factor.restype = ctypes.c_double
        lib.op_ewald_alpha.argtypes = [_f64p, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, _f64p, ctypes.c_int64,
                                       ctypes.c_int, ctypes.c_double, _f64p]
        self.lib = lib

    def keys(self, pos, gridfac, G):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        stride = pos.shape[1]
        out = np.empty(pos.shape[0], dtype=np.uint32)
        self.lib.op_keys(pos.reshape(-1), stride, pos.shape[0], np.float32(gridfac), G, out)
        return out

    def stable_sort(self, keys, nkeys):
        keys = np.ascontiguousarray(keys, dtype=np.uint32)
        sk = np.empty_like(keys)
        perm = np.empty_like(keys)
        self.lib.op_stable_sort(keys, keys.size, nkeys, sk, perm)
        return sk, perm

    def cell_bounds(self, sorted_keys, ncells):
        sk = np.ascontiguousarray(sorted_keys, dtype=np.uint32)
        start = np.empty(ncells, dtype=np.uint32)
        end = np.empty(ncells, dtype=np.uint32)
        self.lib.op_cell_bounds(sk, sk.size, ncells, start, end)
        return start, end

    def shortrange_table(self):
        t = np.empty(1000, dtype=np.float32)
        self.lib.op_shortrange_table(t)
        return t

    def pp(self, pos, params: OpParams, G: int, nthreads: int = 1):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        acc = np.empty_like(pos)
        self.lib.op_pp(pos.reshape(-1), pos.shape[0], ctypes.byref(params), G, nthreads, acc.reshape(-1))
        return acc

    def pp_targets(self, pos, targets, params: OpParams, G: int, nthreads: int = 1):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        tg = np.ascontiguousarray(targets, dtype=np.int64)
        acc = np.zeros_like(pos)
        self.lib.op_pp_targets(pos.reshape(-1), pos.shape[0], tg, tg.size, ctypes.byref(params), G,
                               nthreads, acc.reshape(-1))
        return acc[tg]

    def pair_count(self, pos, params: OpParams, G: int, nthreads: int = 1) -> int:
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        return int(self.lib.op_pair_count(pos.reshape(-1), pos.shape[0], ctypes.byref(params), G,
                                          nthreads))

    def pm(self, pos, params: OpParams, M: int, nthreads: int = 1):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        acc = np.empty_like(pos)
        self.lib.op_pm(pos.reshape(-1), pos.shape[0], ctypes.byref(params), M, nthreads, acc.reshape(-1))
        return acc

    def drift_tables(self, a0, a1, omega0, omega_lambda, hubble, n=1000):
        d = np.empty(n)
        k = np.empty(n)
        self.lib.op_drift_tables(a0, a1, omega0, omega_lambda, hubble, n, d, k)
        return d, k

    def table_factor(self, table, loga0, loga1, tbi, t0, t1):
        table = np.ascontiguousarray(table, dtype=np.float64)
        return self.lib.op_table_factor(table, table.size, loga0, loga1, tbi, t0, t1)

    def ewald(self, src, mass, G, boxsize, softening_h, targets, nthreads=1, alpha_l=0.0):
        """FP64 Ewald-summed periodic force on `targets` from all `src`
        (alpha_l = alpha * L of the split; 0 picks the cheapest)."""
        src = np.ascontiguousarray(src, dtype=np.float64)
        tg = np.ascontiguousarray(targets, dtype=np.float64)
        acc = np.empty_like(tg)
        self.lib.op_ewald_alpha(src.reshape(-1), src.shape[0], mass, G, boxsize, softening_h,
                                tg.reshape(-1), tg.shape[0], nthreads, alpha_l, acc.reshape(-1))
        return acc


class Reference:
    """The reference's own CPU force path for one PMGRID (oracle/_ref/)."""

    def __init__(self, pmgrid: int):
        path = os.path.join(REF_DIR, f"libcucoref_pm{pmgrid}.so")
        if not os.path.isfile(path):
            build_reference((pmgrid,))
        lib = ctypes.CDLL(path)
        lib.cref_begrun.argtypes = [ctypes.c_char_p] + [ctypes.c_double] * 9
        for name in ("cref_G", "cref_hubble", "cref_asmth", "cref_rcut", "cref_timebase_interval",
                     "cref_time", "cref_force_softening"):
            getattr(lib, name).restype = ctypes.c_double
        lib.cref_drift_factor.restype = ctypes.c_double
        lib.cref_kick_factor.restype = ctypes.c_double
        lib.cref_set_pos.argtypes = [_f32p]
        lib.cref_set_vel.argtypes = [_f32p]
        lib.cref_get.argtypes = [ctypes.c_void_p] * 4
        lib.cref_get_tables.argtypes = [_f32p, _f32p]
        lib.cref_simparam.argtypes = [_f32p]
        lib.cref_softparam.argtypes = [_f32p]
        lib.cref_get_timeline.argtypes = [_i32p, _i32p, _i32p]
        lib.cref_set_output.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        self.lib = lib
        self.pmgrid = pmgrid
        assert lib.cref_pmgrid() == pmgrid
        self.n = 0

    def begrun(self, ic, a_max=1.0, soft_comoving=None, soft_maxphys=1e30, max_dloga=0.03,
               errtol=0.025):
        """begrun() with the run's parameters; `ic` is an ics.InitialConditions."""
        from cuco_gb300.ics import write_cuco
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "ic.cuco")
            write_cuco(path, ic)
            c = ic.cosmology
            self.lib.cref_begrun(path.encode(), ic.a, a_max, soft_comoving, soft_maxphys, c.omega0,
                                 c.omega_lambda, c.hubble_param, max_dloga, errtol)
        self.n = int(self.lib.cref_numpart())

    def set_threads(self, n):
        self.lib.cref_set_threads(n)

    def set_pos(self, pos):
        self.lib.cref_set_pos(np.ascontiguousarray(pos, dtype=np.float32).reshape(-1))

    def set_vel(self, vel):
        self.lib.cref_set_vel(np.ascontiguousarray(vel, dtype=np.float32).reshape(-1))

    def get(self):
        out = [np.empty((self.n, 3), dtype=np.float32) for _ in range(4)]
        self.lib.cref_get(*[o.ctypes.data for o in out])
        return out  # pos, vel, acc_pp, acc_pm

    def pp(self, nthreads=1):
        self.lib.cref_pp(nthreads)
        return self.get()[2]

    def pm(self):
        self.lib.cref_pm()
        return self.get()[3]

    def wrap(self):
        self.lib.cref_wrap()

    def step(self, nthreads=1) -> int:
        return int(self.lib.cref_step(nthreads))

    def tables(self):
        d = np.empty(1000, dtype=np.float32)
        k = np.empty(1000, dtype=np.float32)
        self.lib.cref_get_tables(d, k)
        return d, k

    def simparam(self):
        s = np.empty(1009, dtype=np.float32)
        self.lib.cref_simparam(s)
        return s

    def softparam(self):
        s = np.empty(3, dtype=np.float32)
        self.lib.cref_softparam(s)
        return s

    def timeline(self):
        b = np.empty(self.n, dtype=np.int32)
        e = np.empty(self.n, dtype=np.int32)
        pm = np.empty(3, dtype=np.int32)
        self.lib.cref_get_timeline(b, e, pm)
        return b, e, pm

    @property
    def G(self):
        return self.lib.cref_G()

    @property
    def asmth(self):
        return self.lib.cref_asmth()

    @property
    def rcut(self):
        return self.lib.cref_rcut()

    @property
    def softening(self):
        return self.lib.cref_force_softening()

    @property
    def timebase_interval(self):
        return self.lib.cref_timebase_interval()
