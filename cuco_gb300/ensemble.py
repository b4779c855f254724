"""Batched form: many independent boxes stepped together (no counterpart in the
reference).  A thin mirror of the cuco_ensemble_* C ABI (include/cuco_gb300.h):
every phase of a step is one launch over all boxes, and steps after the first
replay one CUDA graph."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from ._native import check
from .engine import BoxConfig


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _configs(configs):
    arr = (_native.CucoConfig * len(configs))()
    for k, c in enumerate(configs):
        arr[k] = c.to_c()
        if c.cell_grid is None:
            arr[k].cell_grid = 0  # autotune
    return arr


class Ensemble:
    def __init__(self, configs: list[BoxConfig]):
        self.lib = _native.load()
        self.cfgs = configs
        self.nbox = len(configs)
        self.h = ctypes.c_void_p()
        check(self.lib.cuco_ensemble_create(_configs(configs), self.nbox, ctypes.byref(self.h)),
              "cuco_ensemble_create")
        self.n = [c.n for c in configs]

    def reshape(self, configs: list[BoxConfig], carry: list[int] | None = None):
        """New set of boxes in the same device arrays; carry[b] = current box
        whose state box b keeps, or -1 (then set it with set_state)."""
        c = None if carry is None else np.ascontiguousarray(carry, dtype=np.int32)
        check(self.lib.cuco_ensemble_reshape(self.h, _configs(configs), len(configs), _ptr(c)),
              "cuco_ensemble_reshape")
        self.cfgs = configs
        self.nbox = len(configs)
        self.n = [x.n for x in configs]

    def close(self):
        if self.h:
            self.lib.cuco_ensemble_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def plan(self, box: int):
        """(cell grid, FFT z-pass row pairs per CTA, axis-pass columns per CTA)"""
        g, p, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self.lib.cuco_ensemble_cell_grid(self.h, box, ctypes.byref(g), ctypes.byref(p), ctypes.byref(b)),
              "cuco_ensemble_cell_grid")
        return g.value, p.value, b.value

    def set_state(self, box: int, pos: np.ndarray, vel: np.ndarray | None = None):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        assert pos.shape == (self.n[box], 3)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float32)
        check(self.lib.cuco_ensemble_set_state(self.h, box, _ptr(pos), _ptr(v)), "cuco_ensemble_set_state")

    def get_state(self, box: int):
        out = [np.empty((self.n[box], 3), dtype=np.float32) for _ in range(4)]
        check(self.lib.cuco_ensemble_get_state(self.h, box, *[_ptr(o) for o in out]), "cuco_ensemble_get_state")
        return out  # pos, vel, acc_pp, acc_pm

    def forces(self):
        check(self.lib.cuco_ensemble_forces(self.h), "cuco_ensemble_forces")

    def step(self, drift, kick_pp, kick_pm=None):
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(drift, dtype=np.float64), (self.nbox,)))
        kp = np.ascontiguousarray(np.broadcast_to(np.asarray(kick_pp, dtype=np.float64), (self.nbox,)))
        km = kp if kick_pm is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(kick_pm, dtype=np.float64), (self.nbox,)))
        check(self.lib.cuco_ensemble_step(self.h, _ptr(d), _ptr(kp), _ptr(km)), "cuco_ensemble_step")

    def sync(self):
        check(self.lib.cuco_ensemble_sync(self.h), "cuco_ensemble_sync")

    def timer_start(self):
        check(self.lib.cuco_ensemble_timer(self.h, 0, None), "cuco_ensemble_timer")

    def timer_stop(self) -> float:
        ms = ctypes.c_float()
        check(self.lib.cuco_ensemble_timer(self.h, 1, ctypes.byref(ms)), "cuco_ensemble_timer")
        return ms.value

    def count_pairs(self, enable: bool) -> int:
        c = ctypes.c_uint64()
        check(self.lib.cuco_ensemble_count_pairs(self.h, int(enable), ctypes.byref(c)), "cuco_ensemble_count_pairs")
        return c.value

    def launches(self) -> int:
        return int(self.lib.cuco_ensemble_launches_per_step(self.h))
