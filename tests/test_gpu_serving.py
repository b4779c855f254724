"""The serving form (cuco_gb300.serve): continuous batching of jobs.

Each job's result must be the same served alone and in a mix of jobs that
arrive and leave while it runs.  Every stage of a step is deterministic (the
stable sort, integer-atomic mass deposit, FFT, interpolation, and a short
range that visits candidates in a fixed order), and a job's state crosses
ensemble rebuilds device to device, so the tolerance is zero: the final
positions and velocities must be bit-identical.  (These jobs run z = 49 -> 0
in a handful of steps, a regime where any rounding difference grows
chaotically, so a tolerance would have to be loose to mean anything.)
Admission respects the HBM budget.  The clock is the server's tick count, so
arrivals are reproducible.
"""
import numpy as np
import pytest

from cuco_gb300 import BoxConfig, ics
from cuco_gb300.engine import MODE_FIXED
from cuco_gb300.serve import Job, Server, footprint

pytestmark = pytest.mark.gpu

# (n_side, box Mpc/h, steps, seed, arrival tick)
JOBS = [(16, 60.0, 6, 11, 0), (20, 90.0, 8, 12, 1), (18, 50.0, 5, 13, 3), (24, 120.0, 9, 14, 4),
        (16, 70.0, 4, 15, 7)]


def make_jobs():
    out = []
    for k, (n_side, L, steps, seed, t) in enumerate(JOBS):
        ic = ics.zeldovich(n_side, L, 49.0, seed)
        cfg = BoxConfig(n=ic.n, pm_grid=2 * n_side, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                        softening=float(np.float32(2.8 * np.float32(0.025 * ic.boxsize / n_side))),
                        mode=MODE_FIXED)
        out.append(Job(k, cfg, ic.pos, ic.canonical_velocity(), ic.a, steps, arrival=float(t)))
    return out


def serve(jobs, budget=1 << 40, bytes_seen=None):
    srv = Server(budget, clock=None)
    srv.clock = lambda: float(srv.ticks)
    peak = [0]
    tick = srv.tick

    def counting_tick():
        r = tick()
        running = [j for j in srv.active if not j.finished]
        peak[0] = max(peak[0], len(running))
        if bytes_seen is not None and srv.active:
            bytes_seen.append(footprint([j.config for j in srv.active]))
        return r

    srv.tick = counting_tick
    done = srv.run(jobs)
    return {j.job_id: j for j in done}, peak[0], srv


def test_each_job_same_alone_and_in_the_mix():
    mix, peak, srv = serve(make_jobs())
    assert len(mix) == len(JOBS) and peak >= 3 and srv.rebuilds >= 4
    for job in make_jobs():
        alone, _, _ = serve([job])
        a, m = alone[job.job_id], mix[job.job_id]
        assert m.done - m.admitted >= job.steps  # it ran all its steps
        assert np.array_equal(m.result_pos, a.result_pos), f"job {job.job_id}: positions differ"
        assert np.array_equal(m.result_vel, a.result_vel), f"job {job.job_id}: velocities differ"


def test_admission_respects_the_hbm_budget():
    jobs = make_jobs()
    sizes = sorted(footprint([j.config]) for j in jobs)
    budget = sizes[-1] + sizes[-2]  # room for the two largest together, not for all
    assert footprint([j.config for j in jobs]) > budget
    seen = []
    done, peak, _ = serve(jobs, budget, seen)
    assert len(done) == len(JOBS)
    assert max(seen) <= budget  # the resident ensemble never exceeded the budget
    assert peak < len(JOBS)
    # every job waited for room or started on arrival, and all finished
    assert all(j.done >= j.arrival for j in done.values())
    # the same results as without a budget: waiting changes no trajectory
    free, _, _ = serve(make_jobs())
    for k, j in done.items():
        assert np.array_equal(j.result_pos, free[k].result_pos)


def test_job_larger_than_the_budget_is_refused():
    jobs = make_jobs()[:1]
    with pytest.raises(RuntimeError):
        serve(jobs, budget=footprint([jobs[0].config]) - 1)
