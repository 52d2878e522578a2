"""The multi-GPU path of bench.py is replicas only: each rank runs its own case, then the
ranks agree on the slowest time. This runs that host-side logic as two gloo ranks on the
CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench

    ws, r, local = bench.dist_env()
    assert (ws, r, local) == (world, rank, rank)
    d = bench.init_dist(ws, "gloo")
    bench.barrier(d)
    t = bench.reduce_max(d, 10.0 + rank)  # each replica's own time
    out[rank] = t
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_replica_time():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        assert dict(out) == {0: 11.0, 1: 11.0}


def test_single_rank_needs_no_process_group():
    import bench

    assert bench.init_dist(1, "gloo") is None
    assert bench.reduce_max(None, 3.5) == 3.5
