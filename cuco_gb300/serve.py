"""Serving form: continuous batching of simulation jobs on one GPU (no
counterpart in the reference, which runs one box per process).

A job is one box run from its initial conditions to a = 1 in its own number
of fixed log-a steps.  The server keeps the state of every admitted job
resident on the device and advances all of them together: each tick is one
step of a batched ensemble (cuco_ensemble_*), every job on its own schedule.
Jobs are admitted first-come first-served while the device bytes of the
running jobs plus the newcomer stay within the HBM budget (and the number of
running jobs within max_active); finished jobs leave.  When the set of running
jobs changes, the ensemble is re-laid out in its own device arrays (which
only grow, so the resident footprint never doubles) and the running jobs'
positions and velocities move device to device, so
a job's trajectory does not depend on who else is running: every stage of a
step is deterministic (stable sort, integer-atomic mass deposit, FFT,
interpolation, a short range that visits candidates in a fixed order), and a
job's result is bit-identical alone and in the mix.

Time comes from a clock callable: wall time for measurements, a tick counter
for tests.  A job's latency is its completion time minus its arrival time.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native
from ._native import check
from .engine import MODE_FIXED, BoxConfig, fixed_step_schedule
from .ensemble import Ensemble


@dataclass
class Job:
    job_id: int
    config: BoxConfig            # mode must match the server's
    pos: np.ndarray              # initial positions (n, 3), float32
    vel: np.ndarray              # initial canonical velocities (n, 3), float32
    a_begin: float
    steps: int                   # fixed log-a steps to a = 1
    arrival: float = 0.0         # in the server clock's units
    # filled in by the server
    drift: np.ndarray = field(default=None, repr=False)
    kick: np.ndarray = field(default=None, repr=False)
    next_step: int = 0           # index into drift/kick (steps + 1 entries)
    admitted: float | None = None
    done: float | None = None
    result_pos: np.ndarray = field(default=None, repr=False)
    result_vel: np.ndarray = field(default=None, repr=False)

    @property
    def finished(self) -> bool:
        return self.next_step > self.steps


def footprint(configs: list[BoxConfig]) -> int:
    """Device bytes an ensemble of these boxes holds (cuco_ensemble_footprint)."""
    lib = _native.load()
    arr = (_native.CucoConfig * max(len(configs), 1))()
    for k, c in enumerate(configs):
        arr[k] = c.to_c()
        if c.cell_grid is None:
            arr[k].cell_grid = 0
    b = ctypes.c_uint64()
    check(lib.cuco_ensemble_footprint(arr, len(configs), ctypes.byref(b)), "cuco_ensemble_footprint")
    return b.value


class Server:
    def __init__(self, hbm_budget: int, max_active: int = 1 << 30, mode: int = MODE_FIXED,
                 clock=time.perf_counter, keep_results: bool = True):
        self.budget = hbm_budget
        self.max_active = max_active
        self.mode = mode
        self.clock = clock
        self.keep_results = keep_results
        self.queue: list[Job] = []       # arrived, waiting
        self.active: list[Job] = []      # resident, in the ensemble's box order
        self.finished: list[Job] = []
        self.ens: Ensemble | None = None
        self.ticks = 0
        self.rebuilds = 0
        self.rebuild_s = 0.0             # host time spent rebuilding ensembles
        self.peak_active = 0             # most jobs running at once
        self.updates = 0                 # particle-updates done

    # -------------------------------------------------------------- intake
    def submit(self, job: Job):
        if job.config.mode != self.mode:
            raise ValueError("job mode differs from the server's")
        _, job.drift, job.kick = fixed_step_schedule(job.a_begin, 1.0, job.steps)
        self.queue.append(job)

    def _admit(self) -> list[Job]:
        new = []
        while self.queue and len(self.active) + len(new) < self.max_active:
            cand = self.active + new + [self.queue[0]]
            if footprint([j.config for j in cand]) > self.budget:
                if not self.active and not new:
                    raise RuntimeError(f"job {self.queue[0].job_id} alone exceeds the HBM budget")
                break
            new.append(self.queue.pop(0))
        return new

    # ------------------------------------------------------------- rebuild
    def _rebuild(self, keep: list[Job], new: list[Job]):
        """Re-lay the ensemble out for the running jobs in the same device
        arrays (they only grow): kept jobs' state moves device to device, new
        jobs' initial conditions are uploaded."""
        t_host = time.perf_counter()
        now = self.clock()
        jobs = keep + new
        if jobs:
            old_index = {id(j): k for k, j in enumerate(self.active)}
            carry = [old_index.get(id(j), -1) for j in jobs]
            if self.ens is None:
                self.ens = Ensemble([j.config for j in jobs])
            else:
                self.ens.reshape([j.config for j in jobs], carry)
            for k, j in enumerate(jobs):
                if carry[k] < 0:
                    self.ens.set_state(k, j.pos, j.vel)
                    j.admitted = now
        self.active = jobs
        self.rebuilds += 1
        self.peak_active = max(self.peak_active, len(jobs))
        self.rebuild_s += time.perf_counter() - t_host

    def _retire(self):
        """Collect finished jobs' results (their boxes stay in the ensemble,
        frozen, until the next rebuild)."""
        now = self.clock()
        for k, j in enumerate(self.active):
            if j.finished and j.done is None:
                if self.keep_results:
                    pos, vel, _, _ = self.ens.get_state(k)
                    j.result_pos, j.result_vel = pos, vel
                j.done = now
                self.finished.append(j)

    # ---------------------------------------------------------------- tick
    def tick(self) -> bool:
        """Admit/retire, then advance every running job one step.  Returns
        False when nothing is running or waiting."""
        self._retire()
        running = [j for j in self.active if not j.finished]
        new = self._admit() if self.queue else []
        if new or len(running) != len(self.active):
            self._rebuild(running, new)
        if not self.active:
            return bool(self.queue)
        nb = len(self.active)
        d = np.zeros(nb)
        kp = np.zeros(nb)
        for k, j in enumerate(self.active):
            if not j.finished:
                d[k], kp[k] = j.drift[j.next_step], j.kick[j.next_step]
        self.ens.step(d, kp, kp)
        for j in self.active:
            if not j.finished:
                j.next_step += 1
                self.updates += j.config.n
        self.ticks += 1
        return True

    def drain(self):
        self.ens and self.ens.sync()
        self._retire()

    def run(self, jobs: list[Job]):
        """Serve jobs whose `arrival` times are in the clock's units, relative
        to the start of the run; returns when all are done."""
        pending = sorted(jobs, key=lambda j: j.arrival)
        t0 = self.clock()
        for j in pending:
            j.arrival += t0
        i = 0
        while i < len(pending) or self.queue or any(not j.finished for j in self.active):
            now = self.clock()
            while i < len(pending) and pending[i].arrival <= now:
                self.submit(pending[i])
                i += 1
            if not self.tick() and i < len(pending):
                # idle: nothing to run until the next arrival
                if self.clock is time.perf_counter:
                    wait = pending[i].arrival - self.clock()
                    if wait > 0:
                        time.sleep(min(wait, 0.01))
                else:
                    self.ticks += 1  # a tick clock moves on by itself
        self.drain()
        if self.ens is not None:
            self.ens.close()
            self.ens = None
        return self.finished

    def close(self):
        if self.ens is not None:
            self.ens.close()
            self.ens = None
