"""Host-side mirror of the reference's force interface over the GB300 engine.

`Box` wraps one resident simulation box of libcuco_gb300.so (cuco_box_t):
positions/velocities in the reference's units and variables (P[].Pos in
kpc/h, P[].Vel = a^2 dx/dt after init.c:30), forces returned like P[].GravAccel
(short range, gravlist.cpp:335-337) and P[].GravPM (long range,
pm_periodic.c:308).  `step()` is one pass of the reference's run loop for a
global timestep (run.c:11-20, timestep.c:26-93): drift, forces, kick.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import _native
from ._native import CucoConfig, Header, check, ptr

HUBBLE = 0.1  # H0 in internal units, km/s per kpc/h (begrun.c:70)
ASMTH = 1.25  # allvars.h:24
RCUT = 4.5    # allvars.h:25

MODE_PLAIN = 0
MODE_FIXED = 1


def reference_split(boxsize: float, pm_grid: int) -> tuple[float, float]:
    """(Asmth, Rcut) with the reference's float rounding (pm_periodic.c:27-28)."""
    b = float(np.float32(boxsize))
    asmth = float(np.float32(ASMTH * b / pm_grid))
    rcut = float(np.float32(RCUT * asmth))
    return asmth, rcut


def cosmo_factors(a0: float, a1: float, omega0: float = 0.3, omega_lambda: float = 0.7,
                  hubble: float = HUBBLE) -> tuple[float, float]:
    """FP64 drift = int da/(H a^3) and kick = int da/(H a^2) (driftfac.c:44-64)."""
    lib = _native.load()
    d = ctypes.c_double()
    k = ctypes.c_double()
    check(lib.cuco_cosmo_factors(a0, a1, omega0, omega_lambda, hubble, ctypes.byref(d),
                                 ctypes.byref(k)), "cuco_cosmo_factors")
    return d.value, k.value


def fixed_step_schedule(a_begin: float, a_end: float, nsteps: int, omega0: float = 0.3,
                        omega_lambda: float = 0.7):
    """Kick-drift-kick factors for `nsteps` equal steps in log a.

    Entry 0 is the opening call (no drift, half kick to the first mid-point), so
    a run is nsteps+1 calls of Box.step; entry s >= 1 drifts a_{s-1} -> a_s and
    kicks a_{s-1/2} -> a_{s+1/2} (the last one closes at a_end), as the
    reference's run loop does for one global power-of-two step
    (timestep.c:48-51: tstart/tend are step mid-points)."""
    la = np.linspace(math.log(a_begin), math.log(a_end), nsteps + 1)
    a = np.exp(la)
    mid = np.exp(0.5 * (la[:-1] + la[1:]))
    drift = np.zeros(nsteps + 1)
    kick = np.zeros(nsteps + 1)
    kick[0] = cosmo_factors(a[0], mid[0], omega0, omega_lambda)[1]
    for s in range(1, nsteps + 1):
        drift[s] = cosmo_factors(a[s - 1], a[s], omega0, omega_lambda)[0]
        hi = mid[s] if s < nsteps else a[nsteps]
        kick[s] = cosmo_factors(mid[s - 1], hi, omega0, omega_lambda)[1]
    return a, drift, kick


@dataclass
class BoxConfig:
    n: int
    pm_grid: int
    boxsize: float
    mass: float
    G: float
    softening: float          # spline length h = 2.8 eps
    cell_grid: int | None = None
    asmth: float | None = None
    rcut: float | None = None
    mode: int = MODE_PLAIN
    device: int = 0

    def to_c(self) -> CucoConfig:
        c = CucoConfig()
        c.n = self.n
        c.pm_grid = self.pm_grid
        c.cell_grid = self.cell_grid or max(self.pm_grid // 4, 8)
        c.boxsize = self.boxsize
        c.mass = self.mass
        c.G = self.G
        c.softening = self.softening
        c.mode = self.mode
        c.device = self.device
        if self.asmth is None or self.rcut is None:
            check(_native.load().cuco_config_reference(ctypes.byref(c)), "cuco_config_reference")
            if self.asmth is not None:
                c.asmth = self.asmth
            if self.rcut is not None:
                c.rcut = self.rcut
        else:
            c.asmth = self.asmth
            c.rcut = self.rcut
        return c


class Box:
    """One resident box on the GPU."""

    PHASES = ("drift+keys", "sort", "reorder", "pm_deposit", "pm_fft", "pm_interp", "shortrange",
              "total")

    def __init__(self, cfg: BoxConfig):
        self.lib = _native.load()
        self.cfg = cfg
        self.c = cfg.to_c()
        self.h = ctypes.c_void_p()
        check(self.lib.cuco_box_create(ctypes.byref(self.c), ctypes.byref(self.h)), "cuco_box_create")
        self.n = cfg.n

    def close(self):
        if self.h:
            self.lib.cuco_box_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, pos: np.ndarray, vel: np.ndarray | None = None):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        assert pos.shape == (self.n, 3)
        v = None
        if vel is not None:
            v = np.ascontiguousarray(vel, dtype=np.float32)
            assert v.shape == (self.n, 3)
        check(self.lib.cuco_box_set_state(self.h, ptr(pos), ptr(v) if v is not None else None, 0),
              "cuco_box_set_state")

    def set_state_fixed(self, pos_u32: np.ndarray, vel: np.ndarray | None = None):
        """Fixed-point boxes: positions as uint32 (units of boxsize / 2^32)."""
        pos = np.ascontiguousarray(pos_u32, dtype=np.uint32)
        assert pos.shape == (self.n, 3)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float32)
        check(self.lib.cuco_box_set_state_fixed(self.h, ptr(pos), ptr(v) if v is not None else None, 0),
              "cuco_box_set_state_fixed")

    def get_state_fixed(self) -> np.ndarray:
        out = np.empty((self.n, 3), dtype=np.uint32)
        check(self.lib.cuco_box_get_state_fixed(self.h, ptr(out), 0), "cuco_box_get_state_fixed")
        return out

    def set_state_device(self, pos_ptr: int, vel_ptr: int | None):
        check(self.lib.cuco_box_set_state(self.h, ctypes.c_void_p(pos_ptr),
                                          ctypes.c_void_p(vel_ptr) if vel_ptr else None, 1),
              "cuco_box_set_state")

    def get_state(self):
        out = [np.empty((self.n, 3), dtype=np.float32) for _ in range(4)]
        check(self.lib.cuco_box_get_state(self.h, *[ptr(o) for o in out], 0), "cuco_box_get_state")
        return out  # pos, vel, acc_pp, acc_pm

    def load_snapshot(self, path: str, initial_conditions: bool = True) -> Header:
        """State from a .cuco IC or snapshot file (read_ic.c:9-45); returns its header."""
        hdr = Header()
        check(self.lib.cuco_box_load_snapshot(self.h, path.encode(), int(initial_conditions),
                                              ctypes.byref(hdr)), "cuco_box_load_snapshot")
        return hdr

    def save_snapshot(self, path: str, header: Header):
        """The state and last forces as a .cuco snapshot (io.c:9-40)."""
        check(self.lib.cuco_box_save_snapshot(self.h, path.encode(), ctypes.byref(header)),
              "cuco_box_save_snapshot")

    def set_softening(self, h: float):
        check(self.lib.cuco_box_set_softening(self.h, h), "cuco_box_set_softening")

    def forces(self, pm: bool = True, pp: bool = True):
        check(self.lib.cuco_box_forces(self.h, int(pm), int(pp)), "cuco_box_forces")

    def step(self, drift: float, kick_pp: float, kick_pm: float | None = None):
        check(self.lib.cuco_box_step(self.h, drift, kick_pp, kick_pp if kick_pm is None else kick_pm),
              "cuco_box_step")

    def run(self, drift, kick_pp, kick_pm=None, a=None, log=None, first_step: int = 0):
        """Steps with the given factors (arrays).  With `log` (a
        steplog.StepLog) every step is timed by phase and logged - each step
        then waits for the one before, so a logged run is not a timed one."""
        n = len(drift)
        if log is not None:
            self.enable_timing(True)
        for k in range(n):
            self.step(drift[k], kick_pp[k], None if kick_pm is None else kick_pm[k])
            if log is not None:
                self.sync()
                t = self.timings()
                rec = {"step": first_step + k, "phase_ms": {p: round(v, 5) for p, v in t.items()},
                       "particle_updates_per_s": self.n / (t["total"] * 1e-3) if t["total"] > 0 else None}
                if a is not None:
                    rec["a"] = float(a[k])
                log.write("box_step", **rec)
        if log is not None:
            self.enable_timing(False)

    def sync(self):
        check(self.lib.cuco_box_sync(self.h), "cuco_box_sync")

    def stream(self) -> int:
        s = ctypes.c_void_p()
        check(self.lib.cuco_box_stream(self.h, ctypes.byref(s)), "cuco_box_stream")
        return s.value or 0

    def enable_timing(self, on: bool = True):
        check(self.lib.cuco_box_enable_timing(self.h, int(on)), "cuco_box_enable_timing")

    def timings(self) -> dict:
        ms = np.zeros(8, dtype=np.float32)
        check(self.lib.cuco_box_timings(self.h, ptr(ms)), "cuco_box_timings")
        return dict(zip(self.PHASES, ms.tolist()))

    def count_pairs(self, enable: bool = True):
        """Count in-range pairs in the short-range launches from now on."""
        check(self.lib.cuco_box_count_pairs(self.h, int(enable)), "cuco_box_count_pairs")

    def pair_count(self, reset: bool = True) -> int:
        c = ctypes.c_uint64()
        check(self.lib.cuco_box_pair_count(self.h, ctypes.byref(c), int(reset)), "cuco_box_pair_count")
        return c.value

    def phase_totals(self, reset: bool = True) -> dict:
        """Per-phase device time summed over the timed steps since the last reset."""
        ms = np.zeros(8, dtype=np.float32)
        check(self.lib.cuco_box_phase_totals(self.h, ptr(ms), int(reset)), "cuco_box_phase_totals")
        return dict(zip(self.PHASES, ms.tolist()))

    def launches(self) -> int:
        return int(self.lib.cuco_box_launches_per_step(self.h))

    def cell_order(self):
        """The short range's source order: (perm_s, slice) per sorted position."""
        perm_s = np.empty(self.n, dtype=np.uint32)
        sl = np.empty(self.n, dtype=np.float32)
        check(self.lib.cuco_box_cell_order(self.h, ptr(perm_s), ptr(sl)), "cuco_box_cell_order")
        return perm_s, sl

    def debug(self):
        n, nc = self.n, self.c.cell_grid ** 3
        keys = np.empty(n, dtype=np.uint32)
        perm = np.empty(n, dtype=np.uint32)
        cs = np.empty(nc, dtype=np.uint32)
        ce = np.empty(nc, dtype=np.uint32)
        check(self.lib.cuco_box_debug(self.h, ptr(keys), ptr(perm), ptr(cs), ptr(ce)), "cuco_box_debug")
        return keys, perm, cs, ce
