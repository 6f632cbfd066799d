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


def test_traffic_summary_matches_the_profile():
    """roofline.traffic is the committed one-pass ncu capture of the gather
    kernel: the mean of its launches' DRAM read + write bytes, above the
    algorithmic 12 E + 20 N + 4 bytes (opinion gathers that miss L2) and
    below the element-touch 20 E + 20 N plus a second read of the 12 E
    bytes of the edge stream."""
    import json
    import bench
    d = json.load(open(os.path.join(os.path.dirname(bench.__file__), "profiles",
                                    "k_opinion_traffic.json")))
    t = bench.traffic_per_launch()
    per = [r + w for r, w in zip(d["dram_bytes_read_per_launch"],
                                 d["dram_bytes_write_per_launch"])]
    assert t == d["bytes_per_launch_full_size"]
    assert abs(t - sum(per) / len(per)) <= 1
    E, N = 200_000_000, 10_000_000
    assert d["algorithmic_bytes_per_launch"] == 12 * E + 20 * N + 4
    assert 12 * E + 20 * N + 4 < t < 20 * E + 20 * N + 12 * E
