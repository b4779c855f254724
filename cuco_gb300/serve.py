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
for tests.  A job's latency is its completion time minus its arrival time;
the completion time is taken after the GPU has finished the job's last step
(the server waits for the ensemble's stream only when a job finishes, not
every tick, so the host prepares the next step while the GPU runs this one).

Output times (run.c:49-59, 75-104; the reference reads them from a list such
as output_32/list_32.txt): a job may list scale factors at which it writes a
snapshot in the reference's .cuco format.  As in the reference, an output
between two steps is a drift of the positions from the last step to the
output time with the velocities as they stand (the last kick), written
without changing the run: the trajectory is the same with or without outputs.

Several processes (one per GPU) share a stream by job: shard_jobs gives each
rank every world-th job in arrival order, with no exchange between ranks.
"""
from __future__ import annotations

import ctypes
import json
import os
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native
from ._native import check
from .engine import MODE_FIXED, Box, BoxConfig, cosmo_factors, fixed_step_schedule
from .ensemble import Ensemble
from .ics import HEADER_DTYPE, PARTICLE_DTYPE


@dataclass
class Job:
    job_id: int
    config: BoxConfig            # mode must match the server's
    pos: np.ndarray              # initial positions (n, 3), float32
    vel: np.ndarray              # initial canonical velocities (n, 3), float32
    a_begin: float
    steps: int                   # fixed log-a steps to a = 1
    arrival: float = 0.0         # in the server clock's units
    outputs: tuple = ()          # scale factors of snapshot outputs (ascending)
    output_dir: str | None = None
    omega0: float = 0.3          # for the snapshot header and the drift to an output
    omega_lambda: float = 0.7
    hubble_param: float = 0.7
    # filled in by the server
    drift: np.ndarray = field(default=None, repr=False)
    kick: np.ndarray = field(default=None, repr=False)
    next_step: int = 0           # index into drift/kick (steps + 1 entries)
    admitted: float | None = None
    done: float | None = None
    result_pos: np.ndarray = field(default=None, repr=False)
    result_vel: np.ndarray = field(default=None, repr=False)
    a: np.ndarray = field(default=None, repr=False)   # scale factor after each step
    snapshots: list = field(default_factory=list)     # paths written, in order
    next_output: int = 0
    cancelled: bool = False
    start_step: int = 0          # a job resumed from a checkpoint starts here
    box: object = field(default=None, repr=False)  # its own Box when it runs outside the ensemble

    @classmethod
    def from_checkpoint(cls, path: str, arrival: float = 0.0) -> "Job":
        """A job resumed from `checkpoint` files: the state of the snapshot,
        the schedule continuing at the step after it."""
        from .ics import read_cuco
        with open(path + ".json") as fh:
            meta = json.load(fh)
        _, parts = read_cuco(path)
        cfg = BoxConfig(**meta["config"])
        return cls(meta["job_id"], cfg, np.ascontiguousarray(parts["Pos"]), np.ascontiguousarray(parts["Vel"]),
                   meta["a_begin"], meta["steps"], arrival=arrival, outputs=tuple(meta["outputs"]),
                   output_dir=meta["output_dir"], start_step=meta["next_step"])

    @property
    def finished(self) -> bool:
        return self.next_step > self.steps


def shard_jobs(jobs: list, rank: int, world: int) -> list:
    """This rank's share of a job stream: every world-th job in arrival order
    (jobs are independent; no data crosses ranks)."""
    order = sorted(range(len(jobs)), key=lambda k: (jobs[k].arrival, k))
    return [jobs[k] for k in order[rank::world]]


def output_positions(pos: np.ndarray, vel: np.ndarray, drift: float, boxsize: float) -> np.ndarray:
    """Positions drifted from the last step to an output time and wrapped into
    [0, L) (predict.c:10-41: Pos += Vel * drift, then the box wrapping)."""
    x = (pos.astype(np.float64) + vel.astype(np.float64) * drift).astype(np.float32)
    L = np.float32(boxsize)
    x = np.where(x < 0, (x.astype(np.float64) + float(L)).astype(np.float32), x)
    x = np.where(x >= L, (x.astype(np.float64) - float(L)).astype(np.float32), x)
    return x


def write_snapshot(path: str, job: Job, a_out: float, pos, vel, acc_pp, acc_pm):
    """HEADER + PARTICLE[] as io.c:9-40 writes them (Ti fields 0: the jobs run
    global steps)."""
    c = job.config
    hdr = np.zeros(1, dtype=HEADER_DTYPE)
    hdr["NumPart"] = c.n
    hdr["Mass"] = c.mass
    hdr["Time"] = a_out
    hdr["Redshift"] = np.float32(1) / np.float32(a_out) - np.float32(1)
    hdr["BoxSize"] = c.boxsize
    hdr["Omega0"], hdr["OmegaLambda"], hdr["HubbleParam"] = job.omega0, job.omega_lambda, job.hubble_param
    parts = np.zeros(c.n, dtype=PARTICLE_DTYPE)
    parts["Pos"], parts["Vel"], parts["Mass"] = pos, vel, c.mass
    parts["GravAccel"], parts["GravPM"] = acc_pp, acc_pm
    with open(path, "wb") as fh:
        fh.write(hdr.tobytes())
        fh.write(parts.tobytes())


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
    """`solo_threshold`: jobs of at least this many particles run on boxes of
    their own (the one-box path, each on its own stream, stepped every tick
    beside the ensemble) instead of in the ensemble: a box that fills the GPU
    by itself gains nothing from batching and runs faster alone.  None keeps
    every job in the ensemble."""

    def __init__(self, hbm_budget: int, max_active: int = 1 << 30, mode: int = MODE_FIXED,
                 clock=time.perf_counter, keep_results: bool = True, log=None, solo_threshold: int | None = None):
        self.budget = hbm_budget
        self.solo_threshold = solo_threshold
        self.solo: list[Job] = []        # running on boxes of their own
        self.max_active = max_active
        self.mode = mode
        self.clock = clock
        self.keep_results = keep_results
        self.log = log                   # a steplog.StepLog: one record per tick and per finished job
        self.queue: list[Job] = []       # arrived, waiting
        self.active: list[Job] = []      # resident, in the ensemble's box order
        self.finished: list[Job] = []
        self.ens: Ensemble | None = None
        self.ticks = 0
        self.rebuilds = 0
        self.rebuild_s = 0.0             # host time spent rebuilding ensembles
        self.peak_active = 0             # most jobs running at once
        self.updates = 0                 # particle-updates done
        self.cancelled_ids: set = set()  # cancelled before they arrived
        self.refused: list[Job] = []     # refused at submission (invalid initial state)

    # -------------------------------------------------------------- intake
    def submit(self, job: Job):
        """Queue a job.  A job whose initial positions or velocities are not
        all finite, or do not match its particle count, is refused (ValueError)
        and recorded in `refused`; nothing already queued or running is
        touched."""
        if job.config.mode != self.mode:
            raise ValueError("job mode differs from the server's")
        n = job.config.n
        pos, vel = np.asarray(job.pos), np.asarray(job.vel)
        if pos.shape != (n, 3) or vel.shape != (n, 3) or not (np.isfinite(pos).all() and np.isfinite(vel).all()):
            job.cancelled = True
            self.refused.append(job)
            raise ValueError(f"job {job.job_id}: initial state is not {n} finite positions and velocities")
        if job.job_id in self.cancelled_ids:
            job.cancelled = True
            job.done = self.clock()
            self.finished.append(job)
            return
        job.a, job.drift, job.kick = fixed_step_schedule(job.a_begin, 1.0, job.steps)
        job.next_step = job.start_step
        while job.next_output < len(job.outputs) and job.outputs[job.next_output] <= job.a[max(job.start_step - 1, 0)]:
            job.next_output += 1  # outputs before a resumed job's state were written before it stopped
        if job.outputs and not job.output_dir:
            raise ValueError("a job with output times needs an output directory")
        self.queue.append(job)

    def cancel(self, job_id) -> None:
        """Cancel a job: a waiting job leaves the queue, a running one stops
        after the step in flight and leaves the ensemble at the next tick (no
        result), a job not yet submitted is dropped when it arrives.  The other
        jobs' trajectories do not change (each job's result is independent of
        the mix)."""
        for j in self.queue:
            if j.job_id == job_id:
                self.queue.remove(j)
                j.cancelled = True
                j.done = self.clock()
                self.finished.append(j)
                return
        for j in self.active + self.solo:
            if j.job_id == job_id and not j.finished:
                j.cancelled = True
                j.next_step = j.steps + 1  # finished: retired without a result
                return
        self.cancelled_ids.add(job_id)

    def checkpoint(self, job_id, path: str) -> None:
        """Write a running job's state: a `.cuco` snapshot at `path` (positions
        after its last step, the velocities as they stand, its last forces)
        and the job's schedule position in `path + ".json"`.  A job made by
        Job.from_checkpoint continues the run where it stands; in the plain
        form it ends bit-identical to the uninterrupted job, in the
        fixed-point form the positions pass through float32 once (about
        1e-7 of the box)."""
        for k, j in list(enumerate(self.active)) + [(None, j) for j in self.solo]:
            if j.job_id == job_id and not j.finished:
                if j.next_step == 0:
                    raise RuntimeError(f"job {job_id} has not run a step yet")
                if k is None:
                    pos, vel, app, apm = j.box.get_state()
                else:
                    self.ens.sync()
                    pos, vel, app, apm = self.ens.get_state(k)
                write_snapshot(path, j, float(j.a[j.next_step - 1]), pos, vel, app, apm)
                c = j.config
                meta = {"job_id": j.job_id, "a_begin": j.a_begin, "steps": j.steps, "next_step": j.next_step,
                        "outputs": list(j.outputs), "output_dir": j.output_dir,
                        "config": {f: getattr(c, f) for f in c.__dataclass_fields__}}
                with open(path + ".json", "w") as fh:
                    json.dump(meta, fh)
                return
        raise KeyError(f"job {job_id} is not running")

    def _is_solo(self, job: Job) -> bool:
        return self.solo_threshold is not None and job.config.n >= self.solo_threshold

    def _admit(self) -> tuple[list[Job], list[Job]]:
        """(new ensemble jobs, new solo jobs) that fit beside the running ones."""
        new, new_solo = [], []
        solo_bytes = sum(footprint([j.config]) for j in self.solo if not j.finished)
        running = len(self.active) + sum(not j.finished for j in self.solo)
        while self.queue and running + len(new) + len(new_solo) < self.max_active:
            job = self.queue[0]
            solo = self._is_solo(job)
            ens_jobs = self.active + new + ([] if solo else [job])
            extra = footprint([job.config]) if solo else 0
            need = (footprint([j.config for j in ens_jobs]) if ens_jobs else 0) + solo_bytes + extra
            if need > self.budget:
                if running == 0 and not new and not new_solo:
                    raise RuntimeError(f"job {job.job_id} alone exceeds the HBM budget")
                break
            (new_solo if solo else new).append(self.queue.pop(0))
            solo_bytes += extra
        return new, new_solo

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
        frozen, until the next rebuild; a solo job's box is released).  A job
        is done when the GPU has run its last step: the stream is waited for
        before the time is taken, only on ticks where a job finishes."""
        for j in [j for j in self.solo if j.finished and j.done is None]:
            j.box.sync()
            if self.keep_results and not j.cancelled:
                pos, vel, _, _ = j.box.get_state()
                j.result_pos, j.result_vel = pos, vel
            j.box.close()
            j.box = None
            self.solo.remove(j)
            self._done(j, self.clock())
        if not any(j.finished and j.done is None for j in self.active):
            return
        self.ens.sync()
        now = self.clock()
        for k, j in enumerate(self.active):
            if j.finished and j.done is None:
                if self.keep_results and not j.cancelled:
                    pos, vel, _, _ = self.ens.get_state(k)
                    j.result_pos, j.result_vel = pos, vel
                self._done(j, now)

    def _done(self, j: Job, now: float):
        j.done = now
        self.finished.append(j)
        if self.log is not None:
            self.log.write("job_done", job=j.job_id, latency=j.done - j.arrival, steps=j.next_step,
                           cancelled=j.cancelled, particles=j.config.n)

    # ---------------------------------------------------------------- tick
    def tick(self) -> bool:
        """Admit/retire, then advance every running job one step.  Returns
        False when nothing is running or waiting."""
        self._retire()
        # before any re-layout: the boxes' last forces are only in place until
        # the ensemble is rebuilt (a rebuild carries positions and velocities)
        self._outputs()
        running = [j for j in self.active if not j.finished]
        new, new_solo = self._admit() if self.queue else ([], [])
        if new or len(running) != len(self.active):
            self._rebuild(running, new)
        for j in new_solo:
            cfg = BoxConfig(**{**j.config.__dict__, "cell_grid": None})
            j.box = Box(cfg)
            j.box.set_state(j.pos, j.vel)
            j.admitted = self.clock()
            self.solo.append(j)
        if new_solo:
            self.peak_active = max(self.peak_active, len(self.active) + len(self.solo))
        if not self.active and not self.solo:
            return bool(self.queue)
        if self.active:
            nb = len(self.active)
            d = np.zeros(nb)
            kp = np.zeros(nb)
            for k, j in enumerate(self.active):
                if not j.finished:
                    d[k], kp[k] = j.drift[j.next_step], j.kick[j.next_step]
            self.ens.step(d, kp, kp)
        for j in self.solo:
            if not j.finished:
                j.box.step(j.drift[j.next_step], j.kick[j.next_step])
        for j in self.active + self.solo:
            if not j.finished:
                j.next_step += 1
                self.updates += j.config.n
        self.ticks += 1
        if self.log is not None:
            self.log.write("tick", tick=self.ticks, time=self.clock(),
                           running=sum(not j.finished for j in self.active + self.solo), queued=len(self.queue),
                           updates=self.updates)
        return True

    def _outputs(self):
        """Snapshots of running jobs whose next step passes an output time:
        step s (s >= 1) drifts a[s-1] -> a[s]; an output a_out in (a[s-1],
        a[s]] is the state after step s-1 drifted to a_out (run.c:49-59).
        Output times at or before the start are skipped."""
        for k, j in list(enumerate(self.active)) + [(None, j) for j in self.solo]:
            s = j.next_step
            if j.finished or not j.outputs or s == 0:
                continue
            while j.next_output < len(j.outputs) and j.outputs[j.next_output] <= j.a[s]:
                a_out = j.outputs[j.next_output]
                if a_out > j.a[0]:
                    pos, vel, app, apm = self.ens.get_state(k) if k is not None else j.box.get_state()
                    drift = cosmo_factors(j.a[s - 1], a_out, j.omega0, j.omega_lambda)[0]
                    path = os.path.join(j.output_dir, f"job{j.job_id}_{j.next_output:03d}.cuco")
                    write_snapshot(path, j, a_out, output_positions(pos, vel, drift, j.config.boxsize), vel,
                                   app, apm)
                    j.snapshots.append(path)
                j.next_output += 1

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
        while i < len(pending) or self.queue or any(not j.finished for j in self.active + self.solo):
            now = self.clock()
            while i < len(pending) and pending[i].arrival <= now:
                try:
                    self.submit(pending[i])
                except ValueError:
                    pass  # refused (recorded in self.refused); the stream goes on
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
        for j in self.solo:
            if j.box is not None:
                j.box.close()
                j.box = None
        self.solo = []
