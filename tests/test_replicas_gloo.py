"""The multi-GPU path is replicas only: every rank renders the same workload
on its own GPU with no collective on the data path; the bench takes the
max-over-ranks time and reports the whole job's rays over it. The host side of
that reduction is checked here with two gloo ranks on the CPU."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    slow = bench.reduce_max(1.5 + rank, dist)  # rank 1 is the slowest
    value = bench.replica_value(4194304, world, slow)
    dist.barrier()
    q.put((rank, slow, value))
    dist.destroy_process_group()


def test_replica_timing_reduction_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]
    assert res[0][2] == pytest.approx(2 * 4194304 / 2.5 / 1e6)


def test_reduce_max_without_process_group():
    import bench
    assert bench.reduce_max(3.25) == 3.25
