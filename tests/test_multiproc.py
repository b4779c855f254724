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
