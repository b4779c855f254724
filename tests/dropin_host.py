"""Drives libcuco_gb300.so's drop-in entry points the way the reference's host
program does: the globals P[], NumPart, header and All are set as begrun()
leaves them (begrun.c:10-27, init.c:8-39), and one pass of run() is restated
from run.c:11-69 (the host program keeps run.c; only the force and integrator
calls go to the library)."""
import ctypes
import math

import numpy as np

from cuco_gb300 import _native, ics
from cuco_gb300._native import All, Header, Particle

TIMEBASE = 1 << 28


class DropIn:
    def __init__(self, pos, vel, mass, boxsize, a_begin, pmgrid, cellgrid, soft_eps, a_max=1.0,
                 errtol=0.025, max_dloga=0.03):
        lib = self.lib = _native.load()
        n = self.n = pos.shape[0]
        self.parts = (Particle * n)()
        raw = self._raw()
        raw[:, 0:3] = pos
        raw[:, 3] = mass
        raw[:, 4:7] = vel
        ctypes.c_void_p.in_dll(lib, "P").value = ctypes.addressof(self.parts)
        ctypes.c_uint.in_dll(lib, "NumPart").value = n
        hdr = Header.in_dll(lib, "header")
        hdr.NumPart, hdr.Mass, hdr.Time, hdr.BoxSize = n, mass, a_begin, boxsize
        al = self.All = All.in_dll(lib, "All")
        al.NumPart, al.BoxSize, al.Mass = n, boxsize, mass
        al.G, al.Hubble = ics.G_INTERNAL, ics.HUBBLE_INTERNAL
        al.Omega0, al.OmegaLambda, al.HubbleParam = 0.3, 0.7, 0.7
        al.Time = al.TimeBegin = a_begin
        al.TimeMax = a_max
        al.Timebase_interval = (math.log(al.TimeMax) - math.log(al.TimeBegin)) / TIMEBASE
        al.Ti_Current = 0
        al.PM_Ti_begstep = al.PM_Ti_endstep = 0
        al.SofteningHalo, al.SofteningHaloMaxPhys = soft_eps, 1e30
        al.ErrTolIntAccuracy, al.MaxSizeTimestep, al.MinSizeTimestep = errtol, max_dloga, 0.0
        al.NumCurrentTiStep = 0
        lib.cuco_dropin_configure(pmgrid, cellgrid)
        lib.set_softenings()
        lib.long_range_init()
        lib.linklist_init()
        lib.init_drift_table()

    def _raw(self):
        return np.ctypeslib.as_array(self.parts).view(np.uint8).reshape(self.n, 60).view(np.float32)

    def _ti(self):
        return np.ctypeslib.as_array(self.parts).view(np.uint8).reshape(self.n, 60)[:, 52:60].view(np.int32)

    def field(self, name):
        sl = {"Pos": slice(0, 3), "Vel": slice(4, 7), "GravAccel": slice(7, 10), "GravPM": slice(10, 13)}[name]
        return self._raw()[:, sl].copy()

    def timeline(self):
        ti = self._ti()
        return ti[:, 1].copy(), ti[:, 0].copy()  # Ti_begstep, Ti_endstep

    def run_pass(self) -> int:
        """run.c:12-20 with no output times."""
        al, lib = self.All, self.lib
        ti_end = self._ti()[:, 0]
        min_glob = int(ti_end.min())
        if min_glob >= al.PM_Ti_endstep:
            min_glob = al.PM_Ti_endstep
        timeold = al.Time
        lib.move_particles(al.Ti_Current, min_glob)
        al.Ti_Current = min_glob
        al.Time = float(np.float32(al.TimeBegin * math.exp(al.Ti_Current * al.Timebase_interval)))
        al.TimeStep = al.Time - timeold
        lib.compute_accelerations()
        lib.advance_and_find_timesteps()
        al.NumCurrentTiStep += 1
        return al.Ti_Current
