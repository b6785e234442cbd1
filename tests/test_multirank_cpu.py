"""The benchmark's multi-rank host logic on CPU: two gloo ranks, each with its
own timing; the job time is the slowest rank's and the job value counts every
rank's replica (weak scaling)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    times = [1.0 + rank, 10.0 - rank]        # rank 0: (1, 10); rank 1: (2, 9)
    got = bench.max_over_ranks(times, dist, "cpu")
    dist.barrier()
    out[rank] = got
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == [2.0, 10.0] and out[1] == [2.0, 10.0]


def test_job_value_counts_every_replica():
    import bench
    assert bench.job_value(4, 432_537_600, 0.01) == pytest.approx(4 * 43.25376)
    assert bench.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]
