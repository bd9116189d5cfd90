"""bench.py's multi-GPU form is replicas only (independent graphs, no data-path
collective); the only cross-rank step is the slowest-rank timing.  Exercised
here with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(0.5 + rank, device="cpu")
    out[rank] = (t, bench.replica_seed(1, rank))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == 1.5
    assert out[0][1] != out[1][1]  # each replica has its own stream


def test_single_process_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(0.25) == 0.25
