"""The N > 1 path of bench.py on CPU: one process per rank over gloo (the
plain path does not shard - each rank runs an independent replica box - so the
only cross-rank work is the barrier and the max over ranks of the timed
region)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.dist_barrier(w)
    t = bench.dist_max(1.0 + rank, w)   # rank 1 is the slowest
    out[rank] = t
    dist.destroy_process_group()


def test_gloo_world2_barrier_and_max_over_ranks():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    assert dict(out) == {0: 2.0, 1: 2.0}


def _shard_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    from types import SimpleNamespace
    from cuco_gb300.serve import shard_jobs
    w, r, _ = bench.dist_setup()
    stream = bench.serving_stream(37)
    jobs = [SimpleNamespace(job_id=sp["id"], arrival=sp["arrival"], n=sp["n_side"] ** 3) for sp in stream]
    mine = shard_jobs(jobs, r, w)
    got = [None] * w
    dist.all_gather_object(got, [j.job_id for j in mine])
    # the aggregate a sharded bench reports: every rank's updates summed
    total = bench.dist_sum(float(sum(j.n for j in mine)), w)
    out[rank] = (got, total, sum(j.n for j in jobs))
    dist.destroy_process_group()


def test_gloo_world2_jobs_sharded_exactly_once():
    """The serving and batched forms split their jobs (boxes) by rank with no
    exchange: over two gloo ranks every job runs on exactly one rank, the
    shares differ by at most one job, and the summed updates are the whole
    stream's."""
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_shard_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    for rank in range(world):
        got, total, whole = out[rank]
        ids = sorted(i for share in got for i in share)
        assert ids == list(range(37))
        assert abs(len(got[0]) - len(got[1])) <= 1
        assert total == whole
