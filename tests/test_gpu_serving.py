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


def test_output_times_write_snapshots_without_changing_the_run(tmp_path):
    """A job with output times (run.c:49-59) served in a mix: its snapshots are
    the state after the step before each output time, drifted to it, in the
    reference's .cuco format; the run itself is the same as without outputs."""
    from cuco_gb300 import fixed_step_schedule
    from cuco_gb300.engine import cosmo_factors
    from cuco_gb300.ensemble import Ensemble
    from cuco_gb300.ics import read_cuco
    from cuco_gb300.serve import output_positions
    jobs = make_jobs()
    target = jobs[3]
    a_sched = fixed_step_schedule(target.a_begin, 1.0, target.steps)[0]
    # between steps, exactly on a step, and the end of the run
    target.outputs = (0.5 * (a_sched[2] + a_sched[3]), float(a_sched[5]), 1.0)
    target.output_dir = str(tmp_path)
    mix, _, _ = serve(jobs)
    j = mix[target.job_id]
    assert len(j.snapshots) == 3
    plain, _, _ = serve(make_jobs())
    assert np.array_equal(j.result_pos, plain[target.job_id].result_pos)
    assert np.array_equal(j.result_vel, plain[target.job_id].result_vel)
    # the same snapshots from the job run alone, step by step
    ref = make_jobs()[3]
    a, drift, kick = fixed_step_schedule(ref.a_begin, 1.0, ref.steps)
    box = Ensemble([ref.config])
    box.set_state(0, ref.pos, ref.vel)
    s = 0
    for path, a_out in zip(j.snapshots, target.outputs):
        while a[s] < a_out:  # run up to the step before the output (states at a[0..s])
            box.step(np.array([drift[s]]), np.array([kick[s]]))
            s += 1
        pos, vel, app, apm = box.get_state(0)
        d = cosmo_factors(float(a[s - 1]), a_out)[0]
        hdr, parts = read_cuco(path)
        assert hdr["Time"] == np.float32(a_out) and int(hdr["NumPart"]) == ref.config.n
        assert np.array_equal(parts["Pos"], output_positions(pos, vel, d, ref.config.boxsize))
        assert np.array_equal(parts["Vel"], vel)
        assert np.array_equal(parts["GravAccel"], app) and np.array_equal(parts["GravPM"], apm)
    box.close()


def test_faults_on_the_host_leave_the_other_jobs_unchanged():
    """Failures made on the host (no GPU fault): a job whose initial state
    carries a NaN is refused at submission, and a running job is cancelled
    mid-run.  Every other job finishes with the result it has alone, bit for
    bit; the cancelled job leaves without a result."""
    jobs = make_jobs()
    bad = jobs[2]
    bad.pos = bad.pos.copy()
    bad.pos[17, 1] = np.nan  # injected into the host-side copy of the state
    import io
    from cuco_gb300 import steplog
    buf = io.StringIO()
    srv = Server(1 << 40, clock=None, log=steplog.StepLog(buf))
    srv.clock = lambda: float(srv.ticks)
    tick = srv.tick

    ran = {}

    def cancelling_tick():
        if srv.ticks == 5:
            ran["steps"] = jobs[1].next_step
            srv.cancel(1)  # job 1 arrived at tick 1 and is running
        return tick()

    srv.tick = cancelling_tick
    done = {j.job_id: j for j in srv.run(jobs)}
    assert [j.job_id for j in srv.refused] == [2] and 2 not in done
    assert done[1].cancelled and done[1].result_pos is None
    assert 0 < ran["steps"] < jobs[1].steps  # it was running and stopped early
    # the structured log: one record per tick, one per finished job
    import json
    recs = [json.loads(x) for x in buf.getvalue().splitlines()]
    assert 0 < sum(r["kind"] == "tick" for r in recs) <= srv.ticks
    finished = {r["job"]: r for r in recs if r["kind"] == "job_done"}
    assert set(finished) == {0, 1, 3, 4} and finished[1]["cancelled"]
    for k in (0, 3, 4):
        alone, _, _ = serve([make_jobs()[k]])
        assert not done[k].cancelled
        assert np.array_equal(done[k].result_pos, alone[k].result_pos)
        assert np.array_equal(done[k].result_vel, alone[k].result_vel)


def test_checkpoint_and_resume(tmp_path):
    """A running job checkpointed (snapshot + schedule position), cancelled,
    and resumed in another server ends bit-identical to the job run without
    interruption (plain form: the state crosses the file exactly)."""
    def plain_jobs():
        out = []
        for j in make_jobs()[:3]:
            cfg = BoxConfig(**{**j.config.__dict__, "mode": 0})
            out.append(Job(j.job_id, cfg, j.pos, j.vel, j.a_begin, j.steps, arrival=0.0))
        return out

    def run(server, jobs, hook=None):
        server.clock = lambda: float(server.ticks)
        if hook:
            tick = server.tick

            def hooked():
                hook(server)
                return tick()
            server.tick = hooked
        return {j.job_id: j for j in server.run(jobs)}

    ref = run(Server(1 << 40, mode=0, clock=None), plain_jobs())
    ck = str(tmp_path / "job1.cuco")

    def stop_job1(server):
        if server.ticks == 4:
            server.checkpoint(1, ck)
            server.cancel(1)

    first = run(Server(1 << 40, mode=0, clock=None), plain_jobs(), stop_job1)
    assert first[1].cancelled
    resumed = Job.from_checkpoint(ck)
    assert 0 < resumed.start_step < resumed.steps
    second = run(Server(1 << 40, mode=0, clock=None), [resumed])
    assert np.array_equal(second[1].result_pos, ref[1].result_pos)
    assert np.array_equal(second[1].result_vel, ref[1].result_vel)
    for k in (0, 2):  # the others were not disturbed
        assert np.array_equal(first[k].result_pos, ref[k].result_pos)


def test_large_jobs_on_boxes_of_their_own():
    """With a solo threshold, the larger jobs run on boxes of their own (the
    one-box path, stepped every tick beside the ensemble): each job's result
    is the same alone and in the mix, and a solo job's result is the one-box
    path's own."""
    from cuco_gb300 import Box, fixed_step_schedule
    threshold = 20 ** 3  # jobs 1 (20^3) and 3 (24^3) go solo

    def run(jobs):
        srv = Server(1 << 40, clock=None, solo_threshold=threshold)
        srv.clock = lambda: float(srv.ticks)
        peak = [0]
        tick = srv.tick

        def counting():
            r = tick()
            peak[0] = max(peak[0], len(srv.solo))
            return r
        srv.tick = counting
        return {j.job_id: j for j in srv.run(jobs)}, peak[0]

    mix, peak_solo = run(make_jobs())
    assert len(mix) == len(JOBS) and peak_solo == 2
    for job in make_jobs():
        alone, _ = run([job])
        assert np.array_equal(mix[job.job_id].result_pos, alone[job.job_id].result_pos)
        assert np.array_equal(mix[job.job_id].result_vel, alone[job.job_id].result_vel)
    j3 = make_jobs()[3]
    _, drift, kick = fixed_step_schedule(j3.a_begin, 1.0, j3.steps)
    box = Box(BoxConfig(**{**j3.config.__dict__, "cell_grid": None}))
    box.set_state(j3.pos, j3.vel)
    for s in range(j3.steps + 1):
        box.step(drift[s], kick[s])
    pos, vel, _, _ = box.get_state()
    box.close()
    assert np.array_equal(mix[3].result_pos, pos) and np.array_equal(mix[3].result_vel, vel)
