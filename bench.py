"""Benchmark: particle-updates/s of full P3M steps on one GB300.

Workload (the plain method at mid size): 128^3 particles in a periodic
256 Mpc/h box, Zel'dovich ICs at z = 49 (P(k) ~ k^0.96 T_BBKS^2, sigma_8 = 0.8,
Omega_m = 0.3, h = 0.7, seeded Philox noise), 256^3 PM mesh, ASMTH = 1.25 mesh
cells, RCUT = 4.5 r_s, spline softening 2.8 * 0.025 of the mean spacing, short
range on a 64^3 cell grid, a z = 49 -> 0 run in 200 equal log-a steps.  A step
is drift + wrap + cell keys + stable radix sort + reorder + PM (deposit, FFT,
Green's function, FD4 gradient, interpolation) + short range + kick.

`value` = N * K / (device time of K consecutive steps), inputs resident in HBM.
The W warm-up steps run from the ICs and the state is then reset to the ICs,
so the timed steps are steps 0..K-1 of the run (K = 200 times the whole run to
z = 0, late steps are the most clustered).  The working set (positions,
velocities, forces, keys, sorted copies, 2 x 64 MB mesh) is ~0.3 GB, above the
129 MB L2, so nothing stays L2-resident from one step to the next.

`e2e` is the same metric through the reference-facing C ABI with host buffers:
the reference's run loop (run.c:11-20) calling the drop-in move_particles,
compute_accelerations and advance_and_find_timesteps on a host P[] array, with
every P[] copy between host and device inside the timed region.

`--impl reference` times full steps of the same run on the CPU force path,
with all host threads: the oracle's C restatement of the reference's CPU code
(bit-exact with the reference's gravlist.cpp + pm_periodic.c built from their
sources; those sources are not on every host, so the restatement is what runs).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time
from types import SimpleNamespace

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SIDE = 128
BOX_MPC = 256.0
PM_GRID = 256
CELL_GRID = 64
Z_INIT = 49.0
NSTEPS_RUN = 200
SEED = 12345
SOFT_FRAC = 0.025
WORKLOAD = "plain-128^3-L256-M256-G64-z49to0-200steps"
MODE = 0  # 0 plain (float32 positions, the reference's arithmetic), 1 fixed point

# --workload presets: (n_side, box Mpc/h, mesh, cell grid, mode, name).  The
# default is the plain method at mid size; the others are the precision form
# (uint32 fixed-point positions) at the same size and both forms at 512^3.
PRESETS = {
    "plain-32": (32, 100.0, 64, 16, 0, "plain-32^3-L100-M64-G16-z49to0-200steps"),
    "precision-32": (32, 100.0, 64, 16, 1, "precision-32^3-L100-M64-G16-z49to0-200steps"),
    "plain-128": (128, 256.0, 256, 64, 0, "plain-128^3-L256-M256-G64-z49to0-200steps"),
    "precision-128": (128, 256.0, 256, 64, 1, "precision-128^3-L256-M256-G64-z49to0-200steps"),
    "plain-512": (512, 1000.0, 1024, 256, 0, "plain-512^3-L1000-M1024-G256-z49to0-200steps"),
    "precision-512": (512, 1000.0, 1024, 256, 1, "precision-512^3-L1000-M1024-G256-z49to0-200steps"),
    "plain-256": (256, 512.0, 512, 128, 0, "plain-256^3-L512-M512-G128-z49to0-200steps"),
    "precision-256": (256, 512.0, 512, 128, 1, "precision-256^3-L512-M512-G128-z49to0-200steps"),
}


BATCHED = "batched-64"
# 256^3 particles as eight 128^3 boxes (L = 256 Mpc/h, M = 256, own seeds): the
# batched fixed-point form against the same boxes on the plain path
BATCHED_256 = "batched-8x128"


def smooth5(n):
    for f in (2, 3, 5):
        while n % f == 0:
            n //= f
    return n == 1


def batched_specs(nbox=64, seed=2024):
    """Boxes of the batched workload: particle grid log-uniform over 16..96 per
    side (rounded to the nearest integer with no prime factor above 5, so the
    2x mesh suits the FFT), L uniform in 50..400 Mpc/h, seeds base+i."""
    rng = np.random.default_rng(seed)
    smooth = [k for k in range(16, 97) if smooth5(k)]
    out = []
    for i in range(nbox):
        x = math.exp(rng.uniform(math.log(16), math.log(96)))
        n_side = min(smooth, key=lambda k: abs(k - x))
        out.append((n_side, 2 * n_side, float(rng.uniform(50.0, 400.0)), seed + 1 + i))
    return out


def batched_256_specs(seed=4096):
    return [(128, 256, 256.0, seed + 1 + i) for i in range(8)]


def run_batched(args, world, rank, local, all_specs=None, workload="batched-64boxes-N16to96-M2N-L50to400-z49"):
    """Many boxes per launch (fixed-point form) against the same boxes stepped
    one at a time on the plain path."""
    from cuco_gb300 import Box, BoxConfig, ics
    from cuco_gb300.engine import MODE_FIXED
    from cuco_gb300.ensemble import Ensemble
    # boxes are independent: rank r takes every world-th box (no exchange)
    all_specs = batched_specs() if all_specs is None else all_specs
    specs = all_specs[rank::world]
    ic_list, cfgs, sched = [], [], None
    for n_side, M, L, seed in specs:
        ic = ics.zeldovich(n_side, L, Z_INIT, seed)
        ic_list.append(ic)
        cfgs.append(BoxConfig(n=ic.n, pm_grid=M, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                              softening=float(np.float32(2.8 * np.float32(SOFT_FRAC * ic.boxsize / n_side))),
                              mode=MODE_FIXED, device=local))
        if sched is None:
            sched = schedule(ic)
    a, drift, kick = sched
    ntot = sum(ic.n for ic in ic_list)
    K, W = args.steps, args.warmup
    t0 = time.perf_counter()
    ens = Ensemble(cfgs)
    setup_s = time.perf_counter() - t0

    def reset():
        for b, ic in enumerate(ic_list):
            ens.set_state(b, ic.pos, ic.canonical_velocity())

    reset()
    for s in range(W):
        ens.step(drift[s], kick[s])
    ens.sync()
    reset()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    dist_barrier(world)
    ens.sync()
    ens.timer_start()
    for s in range(K):
        ens.step(drift[s], kick[s])
    ms = ens.timer_stop()
    ens.sync()
    dist_barrier(world)
    clk = clocks.stop()
    t_total = dist_max(ms / 1e3, world)
    ntot_all = dist_sum(float(ntot), world)
    value = ntot_all * K / t_total
    launches = ens.launches()
    plans = [ens.plan(b) for b in range(len(cfgs))]
    ens.close()
    # the same boxes, one at a time, plain path (default cell grid M/4)
    Kb = min(K, args.baseline_steps)
    t_plain = 0.0
    lib = None
    for ic, c in zip(ic_list, cfgs):
        box = Box(BoxConfig(**{**c.__dict__, "mode": 0, "cell_grid": None}))
        box.set_state(ic.pos, ic.canonical_velocity())
        for s in range(W):
            box.step(drift[s], kick[s])
        box.set_state(ic.pos, ic.canonical_velocity())
        box.sync()
        lib = box.lib
        lib.cuco_box_timer(box.h, 0, None)
        for s in range(Kb):
            box.step(drift[s], kick[s])
        m = ctypes.c_float()
        lib.cuco_box_timer(box.h, 1, ctypes.byref(m))
        t_plain += m.value / 1e3
        box.close()
    plain_rate = ntot_all * Kb / dist_max(t_plain, world)
    sizes = [sp[0] for sp in all_specs]
    line = {
        "metric": "particle-updates/s", "value": value, "unit": "particle-updates/s", "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": 1e3 * t_total / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32", "data": "synthetic",
        "config": {"workload": workload, "boxes": len(all_specs),
                   "particles": int(ntot_all), "n_side_min": min(sizes), "n_side_max": max(sizes),
                   "sharding": f"boxes split by rank ({world} rank(s)), no exchange",
                   "positions": "uint32 fixed point (L/2^32)", "timed_steps": "steps 0..K-1 from z=49",
                   "graph": "one CUDA graph per step, one launch per phase over all boxes"},
        "one_at_a_time_plain": {"value": plain_rate, "unit": "particle-updates/s", "steps": Kb,
                                "ratio": value / plain_rate},
        "autotuned_plans": {"cell_grid": [p[0] for p in plans], "fft_rows_per_cta": [p[1] for p in plans],
                            "fft_cols_per_cta": [p[2] for p in plans]},
        "setup_s": setup_s, "clocks": clk, "gpu_launches": launches * K,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


SERVING = "serving"


def serving_stream(njobs, rate=20.0, seed=5150):
    """Poisson arrivals (exponential gaps, mean 1/rate s); per job: particle
    grid log-uniform over 32..192 per side (nearest integer with no prime
    factor above 5), mesh 2x, L uniform in 50..500 Mpc/h, 50..200 steps, own
    seed."""
    rng = np.random.default_rng(seed)
    smooth = [k for k in range(32, 193) if smooth5(k)]
    t, out = 0.0, []
    for i in range(njobs):
        t += float(rng.exponential(1.0 / rate))
        x = math.exp(rng.uniform(math.log(32), math.log(192)))
        n_side = min(smooth, key=lambda k: abs(k - x))
        out.append({"id": i, "arrival": t, "n_side": n_side, "M": 2 * n_side, "L": float(rng.uniform(50.0, 500.0)),
                    "steps": int(rng.integers(50, 201)), "seed": seed + 1 + i})
    return out


def _serving_ic(spec):
    from cuco_gb300 import ics
    ic = ics.zeldovich(spec["n_side"], spec["L"], Z_INIT, spec["seed"])
    return ic.pos, ic.canonical_velocity(), ic.mass, ic.boxsize, ic.a


def serving_jobs(stream, device=0, mode=0):
    """The stream's jobs with their initial conditions (the request payload),
    made in a spawn process pool before the stream starts."""
    import multiprocessing as mp
    from cuco_gb300 import BoxConfig, ics
    from cuco_gb300.serve import Job
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        ic_data = pool.map(_serving_ic, stream)
    jobs = []
    for sp, (pos, vel, mass, boxsize, a0) in zip(stream, ic_data):
        soft = float(np.float32(2.8 * np.float32(SOFT_FRAC * boxsize / sp["n_side"])))
        cfg = BoxConfig(n=sp["n_side"] ** 3, pm_grid=sp["M"], boxsize=boxsize, mass=mass, G=ics.G_INTERNAL,
                        softening=soft, mode=mode, device=device)
        jobs.append(Job(sp["id"], cfg, pos, vel, a0, sp["steps"], arrival=sp["arrival"]))
    return jobs


def run_serving(args, world, rank, local):
    """Continuous batching of a job stream under an HBM budget, against the
    same jobs run one at a time on the plain path."""
    from cuco_gb300 import Box, BoxConfig, fixed_step_schedule
    from cuco_gb300.engine import MODE_FIXED
    from cuco_gb300.ensemble import Ensemble
    from cuco_gb300.serve import Server
    # the served form in either precision: both meet the rms force error of
    # 1e-3 the serving workload asks for (the plain form 1e-4)
    mode = MODE_FIXED if args.serving_mode == "fixed" else 0
    from cuco_gb300.serve import shard_jobs
    stream = serving_stream(args.jobs)
    # jobs are independent: rank r serves every world-th job (no exchange)
    stream_all = stream
    stream = [vars(sp) for sp in shard_jobs([SimpleNamespace(**sp) for sp in stream_all], rank, world)]
    jobs = serving_jobs(stream, local, mode)
    # autotune every size once (cached), outside the timed stream
    sizes_seen = {}
    for j in jobs:
        sizes_seen.setdefault((j.config.n, j.config.pm_grid), j.config)
    Ensemble(list(sizes_seen.values())).close()
    srv = Server(int(args.hbm_budget_gb * 1e9), max_active=args.max_active, mode=mode, keep_results=False,
                 solo_threshold=args.solo_threshold or None)
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    done = srv.run(jobs)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    lat = np.array([j.done - j.arrival for j in done])
    updates = sum(j.config.n * (j.steps + 1) for j in done)
    wall = dist_max(wall, world)
    updates_all = dist_sum(float(updates), world)
    served_rate = updates_all / wall
    if world > 1:  # latencies of every rank's jobs
        import torch.distributed as dist
        parts = [None] * world
        dist.all_gather_object(parts, lat.tolist())
        lat = np.array([x for p in parts for x in p])
    # one at a time, plain path: a sample of the jobs run alone (their full
    # runs), and a FIFO queue of all jobs at that rate with the same arrivals
    sample = jobs[:: max(1, len(jobs) // args.baseline_jobs)][: args.baseline_jobs]
    plain_t, plain_u = 0.0, 0
    for j in sample:
        box = Box(BoxConfig(**{**j.config.__dict__, "mode": 0, "cell_grid": None}))
        box.set_state(j.pos, j.vel)
        _, drift, kick = fixed_step_schedule(j.a_begin, 1.0, j.steps)
        box.sync()
        t = time.perf_counter()
        for s in range(j.steps + 1):
            box.step(drift[s], kick[s])
        box.sync()
        plain_t += time.perf_counter() - t
        plain_u += j.config.n * (j.steps + 1)
        box.close()
    plain_rate = plain_u / plain_t
    free, fifo = 0.0, []
    for sp in stream_all:
        free = max(free, sp["arrival"]) + sp["n_side"] ** 3 * (sp["steps"] + 1) / plain_rate
        fifo.append(free - sp["arrival"])
    fifo = np.array(fifo)
    sizes = [sp["n_side"] for sp in stream_all]
    line = {
        "metric": "particle-updates/s", "value": served_rate, "unit": "particle-updates/s", "n_gpus": world,
        "steps": int(sum(sp["steps"] + 1 for sp in stream_all)), "warmup": 0, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32+f32" if mode else "f32", "data": "synthetic",
        "config": {"workload": f"serving-{len(stream_all)}jobs-poisson20-N32to192-M2N-L50to500-50to200steps",
                   "jobs": len(stream_all), "arrival_rate_per_s": 20.0, "hbm_budget_gb": args.hbm_budget_gb,
                   "max_active": args.max_active if args.max_active < (1 << 30) else None,
                   "solo_threshold_particles": args.solo_threshold or None,
                   "sharding": f"jobs split by rank ({world} rank(s)), no exchange",
                   "n_side_min": min(sizes), "n_side_max": max(sizes),
                   "positions": "uint32 fixed point (L/2^32)" if mode else "float32",
                   "clock": "host wall time"},
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                      "max": float(lat.max())},
        "wall_s": wall, "particle_updates": int(updates_all), "max_concurrent_jobs": srv.peak_active,
        "rebuilds": srv.rebuilds, "rebuild_s": srv.rebuild_s,
        "one_at_a_time_plain": {"value": plain_rate, "unit": "particle-updates/s", "sample_jobs": len(sample),
                                "fifo_latency_s": {"p50": float(np.percentile(fifo, 50)),
                                                   "p99": float(np.percentile(fifo, 99))},
                                "ratio": served_rate / plain_rate},
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# dram__bytes_read.sum + dram__bytes_write.sum of the short range at z = 49:
# ncu --set full of the first part of the split launch in the first timed step
# of `bench.py --steps 2 --warmup 3 --e2e-steps 0 --no-cpu` (-s 6 -c 1), which
# runs alone under ncu and takes every unit (83.0 + 20.9 MB), and of the
# precision form's (same command with --workload precision-128; 83.3 + 23.1 MB)
SR_TRAFFIC = {"plain-128^3-L256-M256-G64-z49to0-200steps": 103.9e6,
              "precision-128^3-L256-M256-G64-z49to0-200steps": 106.4e6}


# softening (fraction of the mean spacing) of the small box: 0.03, the others 0.025
SOFT_FRACS = {"plain-32": 0.03, "precision-32": 0.03}


def apply_preset(name):
    global N_SIDE, BOX_MPC, PM_GRID, CELL_GRID, MODE, WORKLOAD, SOFT_FRAC
    N_SIDE, BOX_MPC, PM_GRID, CELL_GRID, MODE, WORKLOAD = PRESETS[name]
    SOFT_FRAC = SOFT_FRACS.get(name, SOFT_FRAC)


def workload_config():
    return {"workload": WORKLOAD, "particles": N_SIDE ** 3, "box_mpc_h": BOX_MPC, "pm_grid": PM_GRID,
            "cell_grid": CELL_GRID, "z_init": Z_INIT, "log_a_steps": NSTEPS_RUN, "seed": SEED,
            "softening": f"{SOFT_FRAC} mean spacing",
            "l2": "working set > L2 (no flush)" if N_SIDE >= 128 else
                  "working set < L2, not flushed between steps (a secondary workload, not the headline)",
            "positions": "uint32 fixed point (L/2^32)" if MODE else "float32"}


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_ic():
    from cuco_gb300 import ics
    return ics.zeldovich(N_SIDE, BOX_MPC, Z_INIT, SEED)


def softening_h(ic):
    return float(np.float32(2.8 * np.float32(SOFT_FRAC * ic.boxsize / N_SIDE)))


def schedule(ic):
    from cuco_gb300 import fixed_step_schedule
    return fixed_step_schedule(ic.a, 1.0, NSTEPS_RUN)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def dist_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ----------------------------------------------------------------- CPU arm

def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


class CpuStep:
    """Full steps of the workload on the CPU force path: the oracle's C
    restatement of the reference's CPU code (bit-exact with the reference's own
    gravlist.cpp + pm_periodic.c built from its sources, which is only built
    where those sources are; a host without them runs the restatement).  A step
    is the reference's run-loop body for one global step: drift + wrap
    (predict.c:10-41), the short range of every particle on the reference's
    PMGRID^3 cell grid (gravlist.cpp:117-146,195-338), the full PM
    (pm_periodic.c:67-314, FP64 FFT in place of cuFFT) and the kick
    (timestep.c:56-91)."""

    def __init__(self, nthreads: int):
        import oracle
        from cuco_gb300 import ics
        self.ic = make_ic()
        soft = softening_h(self.ic)
        self.p = oracle.reference_params(self.ic.boxsize, self.ic.mass, ics.G_INTERNAL, PM_GRID, soft)
        self.port = oracle.Port()
        self.kind = "port"
        self.nthreads = nthreads
        _, self.drift, self.kick = schedule(self.ic)
        self.reset()
        self.sample = (f"full steps of the {N_SIDE}^3 workload from z=49: drift+wrap, short range of all "
                       f"{self.ic.n} particles on the reference's {PM_GRID}^3 cell grid, full {PM_GRID}^3 PM, "
                       f"kick; {nthreads} threads")

    def reset(self):
        self.pos = self.ic.pos.astype(np.float32).copy()
        self.vel = self.ic.canonical_velocity().astype(np.float32)
        self.s = 0

    def step(self, targets=None):
        """One step; with `targets`, the short range of those targets only
        (the drift, PM and kick stay whole).  Returns the phase times (s)."""
        s = self.s % (NSTEPS_RUN + 1)
        L = np.float32(self.ic.boxsize)
        t0 = time.perf_counter()
        if self.drift[s]:
            x = self.pos.astype(np.float64) + self.vel.astype(np.float64) * self.drift[s]
            self.pos = np.mod(x, float(L)).astype(np.float32)
            self.pos[self.pos >= L] = 0
        t1 = time.perf_counter()
        if targets is None:
            acc = self.port.pp(self.pos, self.p, PM_GRID, self.nthreads)
        else:
            acc = self.port.pp_targets(self.pos, targets, self.p, PM_GRID, self.nthreads)
        t2 = time.perf_counter()
        apm = self.port.pm(self.pos, self.p, PM_GRID, self.nthreads)
        t3 = time.perf_counter()
        if targets is None:
            self.vel = (self.vel.astype(np.float64) + (acc.astype(np.float64) + apm) * self.kick[s]).astype(
                np.float32)
        t4 = time.perf_counter()
        self.s += 1
        return {"drift_s": t1 - t0, "pp_s": t2 - t1, "pm_s": t3 - t2, "kick_s": t4 - t3, "total_s": t4 - t0}


def cpu_single_core(frac=32):
    """A 1-thread figure on a bounded sample: the short range of a seeded
    1/frac of the targets (scaled by frac) plus the full PM and drift/kick."""
    cs = CpuStep(1)
    rng = np.random.default_rng(7)
    sub = np.sort(rng.choice(cs.ic.n, cs.ic.n // frac, replace=False))
    t = cs.step(sub)
    total = t["drift_s"] + t["pp_s"] * frac + t["pm_s"] + t["kick_s"]
    return {"value": cs.ic.n / total, "unit": "particle-updates/s", "cores": 1,
            "sample": f"one z=49 step on 1 thread: short range of {len(sub)} of {cs.ic.n} targets (x{frac}), "
                      f"full PM and drift/kick"}


def cpu_sample_rate(nthreads: int, steps: int = 2):
    """The GPU arm's cpu_baseline: `steps` full steps from z=49."""
    cs = CpuStep(nthreads)
    t = sum(cs.step()["total_s"] for _ in range(steps))
    return cs.ic.n * steps / t, cs.kind, f"{steps} " + cs.sample, {}


def run_reference_arm(args, world, rank):
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    cs = CpuStep(nthreads)
    for _ in range(args.warmup):
        cs.step()
    cs.reset()  # the timed steps are steps 0..K-1 of the run, as on the GPU arm
    phases = {}
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for k, v in cs.step().items():
            phases[k] = phases.get(k, 0.0) + v
    wall = time.perf_counter() - t0
    val = cs.ic.n * args.steps / wall
    line = {
        "impl": "reference", "metric": "particle-updates/s", "value": val, "unit": "particle-updates/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload_config(),
        "cpu_baseline": {"value": val, "unit": "particle-updates/s", "cores": nthreads, "kind": cs.kind,
                         "sample": f"{args.steps} " + cs.sample, "cpu_model": cpu_model()},
        "e2e": {"value": val, "unit": "particle-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "phase_s_per_step": {k: v / args.steps for k, v in phases.items()},
        "single_core": cpu_single_core(),
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU arm

def measured_hbm_gbs():
    """The HBM copy bandwidth measured on the GB300s the bench runs on
    (MEASURED_PEAKS.json beside this file), else the fallback figure; and
    which."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def step_roofline(n, M, G, pairs_per_step, ms_per_step, fp32_tflops):
    """Whole-step roofline: every phase at its bound (HBM for the sort, deposit,
    transforms and interpolation; the FP32 pipe for the pair force), by the
    fixed algorithmic conventions below, summed and divided by the measured
    step time."""
    hbm, kind = measured_hbm_gbs()
    nbytes = {
        "sort": 28 * n + 8 * G ** 3,                     # pos r + sorted pos w + permutation w; cell bounds
        "deposit": 12 * n + 4 * M ** 3,                  # pos r; density grid w
        "fft": 2 * 2 * 2 * 8 * M * M * (M // 2 + 1),    # fwd + inv, 2 passes each, read + write
        "interpolation": 24 * n + 12 * M ** 3,           # pos r + accel w; three force grids r
    }
    ideal = {k: 1e3 * v / (hbm * 1e9) for k, v in nbytes.items()}
    ideal["pair_force"] = 1e3 * 20.0 * pairs_per_step / (fp32_tflops * 1e12)
    total = sum(ideal.values())
    return {"ideal_ms_per_phase": {k: round(v, 5) for k, v in ideal.items()},
            "algorithmic_bytes": nbytes, "ideal_ms": round(total, 5), "measured_ms": round(ms_per_step, 5),
            "frac": total / ms_per_step, "hbm_peak_gbs": hbm, "hbm_peak_kind": kind,
            "fp32_peak_tflops": fp32_tflops,
            "convention": "bytes per phase as listed (the FD gradient is fused into the interpolation, "
                          "its force grids counted there), 20 FP32 flops per in-range pair"}


def run_gpu_arm(args, world, rank, local):
    from cuco_gb300 import Box, BoxConfig, ics, _native
    lib = _native.load()
    ic = make_ic()
    soft = softening_h(ic)
    a, drift, kick = schedule(ic)
    vel0 = ic.canonical_velocity()
    box = Box(BoxConfig(n=ic.n, pm_grid=PM_GRID, cell_grid=CELL_GRID, boxsize=ic.boxsize,
                        mass=ic.mass, G=ics.G_INTERNAL, softening=soft, device=local, mode=MODE))
    K, W = args.steps, args.warmup
    box.set_state(ic.pos, vel0)
    for s in range(W):
        box.step(drift[s % (NSTEPS_RUN + 1)], kick[s % (NSTEPS_RUN + 1)])
    box.sync()
    box.set_state(ic.pos, vel0)
    box.enable_timing(True)
    pairs = ctypes.c_uint64()
    phase = np.zeros(8)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    dist_barrier(world)
    box.sync()
    lib.cuco_box_timer(box.h, 0, None)
    launches = 0
    for s in range(K):
        box.step(drift[s % (NSTEPS_RUN + 1)], kick[s % (NSTEPS_RUN + 1)])
        launches += box.launches()
    ms = ctypes.c_float()
    lib.cuco_box_timer(box.h, 1, ctypes.byref(ms))
    phase += np.array(list(box.phase_totals().values()))
    box.sync()
    dist_barrier(world)
    clk = clocks.stop()
    t_total = dist_max(ms.value / 1e3, world)
    # in-range pairs of the same K steps, counted in an untimed replay (the
    # counting kernel is a little slower; every stage is deterministic, so the
    # replay visits the same pairs)
    box.enable_timing(False)
    box.set_state(ic.pos, vel0)
    lib.cuco_box_count_pairs(box.h, 1)
    lib.cuco_box_pair_count(box.h, ctypes.byref(pairs), 1)
    for s in range(K):
        box.step(drift[s % (NSTEPS_RUN + 1)], kick[s % (NSTEPS_RUN + 1)])
    lib.cuco_box_pair_count(box.h, ctypes.byref(pairs), 1)
    lib.cuco_box_count_pairs(box.h, 0)
    # the clustered end of the run: steps NSTEPS_RUN-19..NSTEPS_RUN timed after
    # an untimed run from the ICs up to them
    late = None
    if K < NSTEPS_RUN:
        box.set_state(ic.pos, vel0)
        first = NSTEPS_RUN + 1 - 20
        for s in range(first):
            box.step(drift[s], kick[s])
        box.sync()
        box.enable_timing(True)
        box.phase_totals(reset=True)
        lib.cuco_box_timer(box.h, 0, None)
        for s in range(first, NSTEPS_RUN + 1):
            box.step(drift[s], kick[s])
        lm = ctypes.c_float()
        lib.cuco_box_timer(box.h, 1, ctypes.byref(lm))
        late_phase = box.phase_totals()
        box.enable_timing(False)
        t_late = dist_max(lm.value / 1e3, world)
        late = {"steps": f"{first}..{NSTEPS_RUN} of 0..{NSTEPS_RUN} (z = {1 / a[first - 1] - 1:.2f} -> 0)",
                "value": world * ic.n * 20 / t_late, "ms_per_step": 1e3 * t_late / 20,
                "phase_ms_per_step": {k: round(v / 20, 4) for k, v in late_phase.items()}}
    value = world * ic.n * K / t_total
    pp_ms = phase[6] / K
    pair_flops = 20.0 * pairs.value / K
    peak = ctypes.c_double()
    _native.check(lib.cuco_fp32_peak(local, ctypes.byref(peak)), "fp32 peak")
    achieved = pair_flops / (pp_ms * 1e-3) / 1e12
    phases = {k: round(v / K, 4) for k, v in zip(Box.PHASES, phase)}
    line = {
        "metric": "particle-updates/s", "value": value, "unit": "particle-updates/s", "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": 1e3 * t_total / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32" if MODE else "f32", "data": "synthetic",
        "config": workload_config(),
        "roofline": {"bound": "fp32", "kernel": "k_shortrange", "achieved": achieved,
                     "peak": peak.value, "unit": "TFLOP/s", "frac": achieved / peak.value,
                     "traffic": SR_TRAFFIC.get(WORKLOAD),
                     "traffic_note": "DRAM bytes read + written by the short range at z = 49, from an ncu capture "
                                     "of this workload (its split launch's first part, alone under ncu, takes "
                                     "every unit; not measured by this run)",
                     "convention": "20 FP32 flops per in-range pair (pairs counted in-kernel in an untimed replay "
                                   "of the same steps), "
                                   "peak = measured FMA throughput"},
        "step_roofline": step_roofline(ic.n, PM_GRID, CELL_GRID, pairs.value / K, 1e3 * t_total / K,
                                       peak.value),
        "phase_ms_per_step": phases,
        "pairs_per_step": pairs.value / K,
        "late_window": late,
        "clocks": clk,
        "gpu_launches": launches,
    }
    if args.step_log:
        # an untimed pass of the whole run with every step timed by phase and
        # written as one JSON line (each step waits for the one before)
        from cuco_gb300.steplog import StepLog
        box.set_state(ic.pos, vel0)
        log = StepLog(args.step_log)
        box.run(drift, kick, a=a, log=log)
        log.close()
        line["step_log"] = args.step_log
    box.close()
    if args.e2e_steps and MODE == 0:
        line["e2e"] = run_e2e(min(args.e2e_steps, K), ic, soft, local)
    elif MODE:
        line["e2e"] = {"value": None, "reason": "the drop-in C ABI is the plain form only"}
    if rank == 0 and not args.no_cpu:
        try:
            v, kind, sample, info = cpu_sample_rate(os.cpu_count() or 1)
            line["cpu_baseline"] = {"value": v, "unit": "particle-updates/s",
                                    "cores": os.cpu_count(), "kind": kind, "sample": sample,
                                    "cpu_model": cpu_model()}
        except Exception as e:  # the CPU baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "error": str(e)}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_e2e(steps, ic, soft, device):
    """The reference's run loop (run.c:11-20) over the drop-in C ABI with a host
    P[] array: every call reads P[] from the host and writes its results back
    (in place over the host link where the device reads pageable host memory,
    else through a device mirror), with the host time of each call."""
    from cuco_gb300 import _native, ics
    from cuco_gb300._native import All, Header, Particle
    lib = _native.load()
    n = ic.n
    parts = (Particle * n)()
    raw = np.ctypeslib.as_array(parts).view(np.uint8).reshape(n, 60).view(np.float32)
    raw[:, 0:3] = ic.pos
    raw[:, 3] = ic.mass
    raw[:, 4:7] = ic.canonical_velocity()
    ti = np.ctypeslib.as_array(parts).view(np.uint8).reshape(n, 60)[:, 52:60].view(np.int32)
    ti[:] = 0
    ctypes.c_void_p.in_dll(lib, "P").value = ctypes.addressof(parts)
    ctypes.c_uint.in_dll(lib, "NumPart").value = n
    hdr = Header.in_dll(lib, "header")
    hdr.NumPart, hdr.Mass, hdr.Time, hdr.BoxSize = n, ic.mass, ic.a, ic.boxsize
    al = All.in_dll(lib, "All")
    al.NumPart, al.BoxSize, al.Mass = n, ic.boxsize, ic.mass
    al.G, al.Hubble = ics.G_INTERNAL, ics.HUBBLE_INTERNAL
    al.Omega0, al.OmegaLambda, al.HubbleParam = 0.3, 0.7, 0.7
    al.Time = al.TimeBegin = ic.a
    al.TimeMax = 1.0
    al.Timebase_interval = (math.log(1.0) - math.log(float(np.float32(ic.a)))) / (1 << 28)
    al.Ti_Current = 0
    al.PM_Ti_begstep = al.PM_Ti_endstep = 0
    eps = np.float32(SOFT_FRAC * ic.boxsize / N_SIDE)
    al.SofteningHalo, al.SofteningHaloMaxPhys = eps, 1e30
    # every particle on the PM step: the acceleration criterion never binds
    al.ErrTolIntAccuracy = 1e30
    al.MaxSizeTimestep = (math.log(1.0) - math.log(ic.a)) / NSTEPS_RUN
    al.MinSizeTimestep = 0.0
    lib.cuco_dropin_configure(PM_GRID, CELL_GRID)
    lib.set_softenings()
    lib.long_range_init()
    lib.linklist_init()
    lib.init_drift_table()

    calls = {"sync_point": 0.0, "move_particles": 0.0, "compute_accelerations": 0.0,
             "advance_and_find_timesteps": 0.0}

    def one_step():
        # find_next_sync_point_and_drift (run.c:28-69) with no output times; the
        # scan of P[].Ti_endstep (run.c:35-40) is the library's, which returns
        # the minimum advance_and_find_timesteps computed on the device.  Each
        # call returns with its work done (P[] updated), so host time per call
        # is its cost.
        t = [time.perf_counter()]
        min_glob = lib.cuco_dropin_min_ti_endstep()
        if min_glob >= al.PM_Ti_endstep:
            min_glob = al.PM_Ti_endstep
        t.append(time.perf_counter())
        lib.move_particles(al.Ti_Current, min_glob)
        al.Ti_Current = min_glob
        al.Time = float(al.TimeBegin * math.exp(al.Ti_Current * al.Timebase_interval))
        t.append(time.perf_counter())
        lib.compute_accelerations()
        t.append(time.perf_counter())
        lib.advance_and_find_timesteps()
        t.append(time.perf_counter())
        for k, name in enumerate(calls):
            calls[name] += t[k + 1] - t[k]

    one_step()  # opening force + half kick (untimed warm-up)
    one_step()
    for name in calls:
        calls[name] = 0.0
    t0 = time.perf_counter()
    for _ in range(steps):
        one_step()
    dt = time.perf_counter() - t0
    if lib.cuco_dropin_host_access():
        # kernels stream whole 60-byte records of P[] over the host link:
        # each of the three calls reads P[] once and writes it once
        # (compute_accelerations through the device mirror)
        h2d, d2h, access = 3 * 60 * n, 3 * 60 * n, "kernels stream P[] records in place over the host link"
    else:
        h2d, d2h, access = 3 * 60 * n, 3 * 60 * n, "whole P[] copied in and out per call"
    return {"value": n * steps / dt, "unit": "particle-updates/s",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": steps, "path": "drop-in run loop: move_particles + compute_accelerations + "
                                    "advance_and_find_timesteps on host P[] (" + access + ")",
            "calls_ms_per_step": {k: round(v * 1e3 / steps, 4) for k, v in calls.items()},
            "link": link_bandwidth(60 * n, device)}


def link_bandwidth(nbytes, device, reps=5):
    """GB/s of one plain cudaMemcpyAsync of `nbytes` from pinned host memory to
    the device and back (CUDA events, best of `reps`): the host link's copy
    rate that the drop-in's P[] traffic is measured against."""
    import torch
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    dev = torch.empty(nbytes, dtype=torch.uint8, device=device)
    out = {}
    for name, (dst, src) in (("h2d_pinned_gbs", (dev, host)), ("d2h_pinned_gbs", (host, dev))):
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1) * 1e-3)
        out[name] = round(nbytes / best / 1e9, 1)
    out["bytes"] = nbytes
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=NSTEPS_RUN)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--step-log", default=None,
                    help="write an untimed pass of the whole run, one JSON line per step with phase times")
    ap.add_argument("--workload", default="plain-128", choices=sorted(PRESETS) + [BATCHED, BATCHED_256, SERVING])
    ap.add_argument("--baseline-steps", type=int, default=20)
    ap.add_argument("--jobs", type=int, default=120, help="serving: jobs in the stream")
    ap.add_argument("--baseline-jobs", type=int, default=8, help="serving: jobs run alone on the plain path")
    ap.add_argument("--hbm-budget-gb", type=float, default=150.0)
    ap.add_argument("--solo-threshold", type=int, default=0,
                    help="serving: jobs of at least this many particles run on boxes of their own (0: none)")
    ap.add_argument("--max-active", type=int, default=1 << 30,
                    help="serving: most jobs running at once (besides the HBM budget)")
    ap.add_argument("--serving-mode", default="plain", choices=["plain", "fixed"],
                    help="serving: precision of the served ensemble")
    args = ap.parse_args()
    if args.workload == SERVING:
        world, rank, local = dist_setup()
        run_serving(args, world, rank, local)
        return
    if args.workload in (BATCHED, BATCHED_256):
        args.warmup = max(args.warmup, 3)
        world, rank, local = dist_setup()
        if args.workload == BATCHED:
            run_batched(args, world, rank, local)
        else:
            run_batched(args, world, rank, local, batched_256_specs(), "batched-8x128^3-L256-M256-z49")
        return
    apply_preset(args.workload)
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
    else:
        run_gpu_arm(args, world, rank, local)


if __name__ == "__main__":
    main()
