"""The multi-GPU form of the benchmark is replicas only: every rank runs its
own simulation, the job's time is the slowest rank's, and the whole-job
throughput is world size x the units of one replica over that time.  The
host side of this is checked here with two gloo ranks on the CPU."""
import os
import socket

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


def test_reference_arm_line_on_cpu():
    """`bench.py --impl reference` (the oracle's C restatement on the host
    cores, no GPU) prints one JSON line with the contract's fields: the
    reference tag, a cpu_baseline describing the run, and an e2e block with
    no host-device copies."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                        "--n", "20000", "--steps", "2", "--warmup", "1", "--cpu-seconds", "1"],
                       capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "edge-updates/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["workload"] == "bounded_confidence_opinion_chung_lu"

