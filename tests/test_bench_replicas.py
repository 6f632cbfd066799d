"""The multi-GPU form of the benchmark is replicas only: every rank runs its
own simulation, the job's time is the slowest rank's, and the whole-job
throughput is world size x the units of one replica over that time.  The
host side of this is checked here with two gloo ranks on the CPU."""
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
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        t = [1.5, 2.5][rank]  # seconds this replica took
        slowest = bench.max_over_ranks(t)
        value = bench.job_throughput(world, 1000.0, slowest)
        dist.barrier()
        q.put((rank, slowest, value))
    finally:
        dist.destroy_process_group()


def test_replica_timing_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2.5, 2.5]        # every rank sees the slowest time
    assert [o[2] for o in out] == [800.0, 800.0]    # 2 x 1000 units / 2.5 s


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks(3.0) == 3.0
    assert bench.job_throughput(1, 10.0, 2.0) == 5.0
