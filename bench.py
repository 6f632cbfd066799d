#!/usr/bin/env python
"""Benchmark of the GB300 transition step (apply! of Vahana.jl).

Headline workload: bounded-confidence opinion dynamics, Opinion{x::Float64}
with N = 10^7 agents on a directed Chung-Lu graph (exponent 2.5, mean
in-degree 20, expected degree capped at 10^4, E = 2*10^8 edges with Float64
weights), all inputs synthetic and seeded (Philox4x32-10).  One bench step is
one apply!(sim, bounded_confidence, Opinion, [Opinion, Weight], Opinion).

  value  edge-updates/s with the state resident in HBM (CUDA events on the
         simulation's stream around K steps; inputs are larger than L2).
  e2e    the same metric through the C ABI with host buffers: each step
         uploads the opinions from pinned host memory (vg_write_agents),
         runs apply! and reads the new opinions back (vg_read_agents).
  roofline  algorithmic bytes of one launch of the gather kernel,
         12 E + 20 N + 4 (4 B source index + 8 B weight per edge, row
         pointers, opinion read and write), over its CUDA-event duration,
         against the measured HBM copy bandwidth.
  parity the model's 50 steps from the initial state on the GPU against the
         oracle's C restatement on the same graph: rows up to the hub
         threshold bit-exact after one step, every row within 1e-12 relative
         after 50 steps, and the ordered path (no hub split) bit-exact after
         50 steps.
  cpu_baseline  the oracle's 50 steps of that comparison (OpenMP over all
         host cores), timed.
  secondary  the other workloads, each in its own process, each with its own
         parity check: SIR (N = 10^5, 100 steps), Life B3/S23 on 4096^2 cells
         with 10^6 walkers (1000 steps), the batched ensemble of 512 SIR
         instances and the serving stream (1024 jobs at 10 and 1000 jobs/s).

--impl reference times that CPU restatement alone on this workload (the
reference itself is Julia, which neither machine has).
Multi-GPU: replicas only (one independent simulation per rank).
"""
import argparse
import numpy as np
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "vahana.jl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "edge-updates/s"
WORKLOAD = "bounded_confidence_opinion_chung_lu"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=10_000_000)
    ap.add_argument("--mean-degree", type=float, default=20.0)
    ap.add_argument("--wmax", type=float, default=1e4)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--hub-threshold", type=int, default=1536)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="opinion",
                    choices=["opinion", "batch", "serve", "sir", "life", "fp64"])
    ap.add_argument("--secondary", default="sir,life,batch,serve",
                    help="opinion workload: the other workloads run afterwards, each in "
                         "its own process ('none': no other workload)")
    ap.add_argument("--no-parity", action="store_true",
                    help="opinion workload: skip the 50-step oracle comparison")
    ap.add_argument("--jobs", type=int, default=512)
    ap.add_argument("--rates", default="100,1000")
    ap.add_argument("--serve-budget-gb", type=float, default=64.0)
    ap.add_argument("--plain-sample", type=int, default=24)
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--batch-steps", type=int, default=200)
    ap.add_argument("--batch-warmup-instances", type=int, default=8,
                    help="batch workload: instances of the warm-up batch built first (0: none)")
    ap.add_argument("--model-steps", type=int, default=0,
                    help="sir/life workloads: timed steps (default: the model's 100 / 1000)")
    return ap.parse_args()


def config(args):
    return {"workload": WORKLOAD, "agents": args.n, "edges": int(round(args.mean_degree * args.n)),
            "mean_in_degree": args.mean_degree, "degree_exponent": 2.5,
            "max_expected_degree": args.wmax, "eps": 0.3, "mix": 0.5,
            "model_steps_reference": 50, "l2": "inputs larger than L2 (2.6 GB per step)",
            "parallelism": "replicas"}


# ---------------------------------------------------------------- helpers
class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_launch():
    """DRAM bytes per launch of the gather kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "k_opinion_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("bytes_per_launch_full_size")
    return None


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, device="cpu"):
    """The largest x over all ranks (a job's time is its slowest replica's);
    x itself when no process group is running or it has one rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world_size, units_per_rank, seconds):
    """Whole-job units per second: every replica processes units_per_rank in
    the job's time (the maximum over the ranks)."""
    return world_size * units_per_rank / seconds


# ------------------------------------------------------------- CPU legs
NO_SPLIT = 4294967295  # hub threshold that keeps every row on the ordered path
PARITY_STEPS = 50       # the model's step count for the opinion workload
PARITY_RTOL = 1e-12     # stated tolerance where hub rows regroup their sums


def oracle_graph(vh, models, run):
    """The oracle's own per-target containers, built from the edge records
    staged before finish_init! (in add_edge! call order): (row_ptr, src, w)
    with w in container order."""
    from oracle import models as om
    frm, to, pl = models.staged_edges(run.sim, "Weight")
    g = om.build_inedges(run.n, frm, to)
    del frm, to
    w_in = np.ascontiguousarray(pl["w"][g[2]])
    return g[0], g[1], w_in


def max_rel_err(got, ref):
    """Largest |got - ref| / |ref| over the entries whose bits differ."""
    diff = got.view(np.uint64) != ref.view(np.uint64)
    if not diff.any():
        return 0.0
    g, r = got[diff], ref[diff]
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.abs(g - r) / np.abs(r)
    rel[~np.isfinite(rel)] = np.inf
    return float(rel.max())


def opinion_parity(vh, run, g, x_init, hub_thr, steps=PARITY_STEPS):
    """The model's `steps` steps from the initial state on the GPU, once with
    the hub split at hub_thr (the timed configuration) and once on the
    ordered path, against the oracle's C restatement on its own containers
    of the same edges.  Returns (parity record, oracle steps, oracle seconds,
    oracle threads)."""
    from oracle import models as om
    rp, src, w = g
    threads = om.threads()
    x = x_init.copy()
    t0 = time.perf_counter()
    for k in range(steps):
        x = om.opinion_step((rp, src, None), w, x, 0.3, 0.5, 0.5, nthreads=threads)
        if k == 0:
            ref1 = x.copy()
    t_cpu = time.perf_counter() - t0
    ref = x
    m = run.model

    def gpu_steps(thr, k):
        for _ in range(k):
            vh.apply_(run.sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"],
                      ["Opinion"], params=[m["Weight"].index, 0.3, 0.5, 0.5, thr])
        vh.synchronize(run.sim)
        return vh.read_agents(run.sim, "Opinion")[0]["x"].copy()

    vh.write_agents(run.sim, "Opinion", x=x_init)
    g1 = gpu_steps(hub_thr, 1)
    gk = gpu_steps(hub_thr, steps - 1)
    vh.write_agents(run.sim, "Opinion", x=x_init)
    ok = gpu_steps(NO_SPLIT, steps)
    deg = np.diff(rp.astype(np.int64))
    hub = deg > hub_thr
    b = lambda a: a.view(np.uint64)
    low_exact = int((b(g1)[~hub] == b(ref1)[~hub]).sum())
    split = {"hub_threshold": int(hub_thr), "hub_rows": int(hub.sum()),
             "step1_rows_at_or_below_threshold": int((~hub).sum()),
             "step1_rows_at_or_below_threshold_bit_exact": low_exact,
             "step1_hub_rows_max_rel_err": max_rel_err(g1[hub], ref1[hub]),
             "final_rows_bit_exact": int((b(gk) == b(ref)).sum()),
             "final_max_rel_err": max_rel_err(gk, ref)}
    ordered = {"final_rows_bit_exact": int((b(ok) == b(ref)).sum()),
               "final_max_rel_err": max_rel_err(ok, ref)}
    n = int(x_init.size)
    passed = (low_exact == split["step1_rows_at_or_below_threshold"]
              and split["step1_hub_rows_max_rel_err"] <= PARITY_RTOL
              and split["final_max_rel_err"] <= PARITY_RTOL
              and ordered["final_rows_bit_exact"] == n)
    rec = {"steps": steps, "rows": n, "from": "initial state", "rtol": PARITY_RTOL,
           "oracle": "oracle/models.c on containers built from the staged edge records",
           "split": split, "ordered": ordered, "pass": bool(passed)}
    return rec, steps, t_cpu, threads


def cpu_graph_host(args):
    """The same graph built on the host by the oracle's generator."""
    from oracle import models as om
    n = args.n
    e = int(round(args.mean_degree * n))
    frm, to, w = om.gen_chung_lu(n, e, args.mean_degree, 2.5, args.wmax, args.seed)
    g = om.build_inedges(n, frm, to)
    del frm, to
    import numpy as np
    w_in = np.ascontiguousarray(w[g[2]])
    return g[0], g[1], w_in


def time_cpu(g, x0, max_seconds):
    """Run the oracle's step until max_seconds have passed (at least one)."""
    from oracle import models as om
    rp, src, w = g
    threads = om.threads()
    x = x0.copy()
    steps, t0 = 0, time.perf_counter()
    while True:
        x = om.opinion_step((rp, src, None), w, x, 0.3, 0.5, 0.5, nthreads=threads)
        steps += 1
        el = time.perf_counter() - t0
        if el >= max_seconds or steps >= 50:
            break
    return steps, el, threads


# ----------------------------------------------------------------- arms
def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from vahana_gb300 import models
    from oracle import models as om
    g = cpu_graph_host(args)
    x0 = models.opinion_initial_state(args.n, args.seed)
    e = int(g[0][-1])
    # one warm-up step, then timed full steps (each one bounded sample of the
    # workload) until --cpu-seconds have passed or --steps are done
    time_cpu(g, x0, 0.0)
    threads = om.threads()
    times, x, t_all = [], x0, time.perf_counter()
    while len(times) < max(1, args.steps):
        t0 = time.perf_counter()
        x = om.opinion_step((g[0], g[1], None), g[2], x, 0.3, 0.5, 0.5, nthreads=threads)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > args.cpu_seconds:
            break
    ms = 1e3 * sum(times) / len(times)
    v = e / (ms * 1e-3)
    out = {"metric": METRIC, "value": v, "unit": "edge-updates/s", "n_gpus": args.gpus,
           "steps": len(times), "warmup": 1, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference", "config": config(args),
           "cpu_baseline": {"value": v, "unit": "edge-updates/s", "cores": threads,
                            "kind": "port",
                            "sample": "%d full steps of the oracle's C restatement (OpenMP) "
                                      "on the same graph" % len(times)},
           "e2e": {"value": v, "unit": "edge-updates/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_ours(args):
    import numpy as np
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    import vahana_gb300 as vh
    from vahana_gb300 import models
    vh.build()
    stream = torch.cuda.Stream()
    run = models.build_opinion(n=args.n, mean_degree=args.mean_degree, wmax=args.wmax,
                               seed=args.seed, stream=stream.cuda_stream,
                               hub_threshold=args.hub_threshold)
    check_parity = rank == 0 and ws == 1 and not args.no_parity
    x_init = vh.read_agents(run.sim, "Opinion")[0]["x"].copy()
    g_oracle = oracle_graph(vh, models, run) if check_parity else None
    vh.finish_init(run.sim)
    vh.set_async(run.sim, True)
    E, N = run.nedges, run.n
    for _ in range(args.warmup):
        run.step()
    vh.synchronize(run.sim)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # ---- device-resident timed region
    K = args.steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(K)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk = Clocks(local)
    barrier()
    torch.cuda.synchronize()
    clk.start()
    time.sleep(0.3)
    start.record(stream)
    for k in range(K):
        ev[k][0].record(stream)
        run.step()
        ev[k][1].record(stream)
    end.record(stream)
    vh.synchronize(run.sim)
    torch.cuda.synchronize()
    clocks = clk.stop()
    barrier()
    total_ms = start.elapsed_time(end)
    kernel_ms = sorted(a.elapsed_time(b) for a, b in ev)
    mean_kernel_ms = sum(kernel_ms) / len(kernel_ms)
    total_ms = max_over_ranks(total_ms, "cuda")
    value = job_throughput(ws, E * K, total_ms * 1e-3)

    # ---- end to end through the C ABI with pinned host buffers: every step
    # uploads the opinions from host memory and returns the new ones there
    # (vg_apply_host: the download of finished row ranges overlaps the
    # gather); beside it the same step as three calls (vg_write_agents,
    # vg_apply, vg_read_agents), copies and kernel one after the other
    Ke = args.e2e_steps
    xh = torch.empty(N, dtype=torch.float64, pin_memory=True)
    xo = torch.empty(N, dtype=torch.float64, pin_memory=True)
    xh.numpy()[:] = vh.read_agents(run.sim, "Opinion")[0]["x"]
    import ctypes as C
    from vahana_gb300._lib import lib, check
    from vahana_gb300.api import _apply_args
    tn = run.model["Opinion"].index
    inp = (C.c_void_p * 1)(xh.data_ptr())
    outp = (C.c_void_p * 1)(xo.data_ptr())
    nout = C.c_uint64()
    hargs = _apply_args(run.sim, "bounded_confidence", ["Opinion"], ["Opinion", "Weight"],
                        ["Opinion"], (), None,
                        [run.model["Weight"].index, 0.3, 0.5, 0.5, args.hub_threshold])

    def e2e_step():
        check(lib().vg_apply_host(run.sim._h, *hargs, tn, inp, outp, N))

    def e2e_serial_step():
        check(lib().vg_write_agents(run.sim._h, tn, inp, N))
        run.step()
        check(lib().vg_read_agents(run.sim._h, tn, outp, None, N, C.byref(nout)))

    def e2e_time(fn):
        fn()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(Ke):
            fn()
        torch.cuda.synchronize()
        return max_over_ranks(time.perf_counter() - t0, "cuda")
    e2e_s = e2e_time(e2e_step)
    serial_s = e2e_time(e2e_serial_step)
    e2e = {"value": job_throughput(ws, E * Ke, e2e_s), "unit": "edge-updates/s",
           "h2d_bytes_per_step": 8 * N, "d2h_bytes_per_step": 8 * N,
           "call": "vg_apply_host (pinned host buffers)", "ms_per_step": 1e3 * e2e_s / Ke,
           "three_calls": {"value": job_throughput(ws, E * Ke, serial_s),
                           "ms_per_step": 1e3 * serial_s / Ke,
                           "call": "vg_write_agents + vg_apply + vg_read_agents"}}

    # ---- roofline of the gather kernel
    alg_bytes = 12 * E + 20 * N + 4
    peak, kind = peaks()
    achieved = alg_bytes / (mean_kernel_ms * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": kind, "traffic": traffic_per_launch(),
            "algorithmic_bytes_per_launch": alg_bytes, "kernel": "k_opinion",
            "kernel_ms_mean": mean_kernel_ms, "kernel_ms_median": kernel_ms[len(kernel_ms) // 2]}
    # every gathered opinion counted (8 B per edge more): reported beside, not the target
    touch_bytes = 20 * E + 20 * N
    roof["element_touch_bytes_per_launch"] = touch_bytes
    roof["element_touch_gbs"] = touch_bytes / (mean_kernel_ms * 1e-3) / 1e9

    out = {"metric": METRIC, "value": value, "unit": "edge-updates/s", "n_gpus": ws,
           "steps": K, "warmup": args.warmup, "ms_per_step": total_ms / K,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": config(args), "e2e": e2e, "roofline": roof,
           "clocks": clocks, "gpu_launches": K}

    # ---- parity at the model's size and step count, and the CPU baseline
    # (rank 0, N = 1 only): the oracle's 50 steps of the comparison, timed
    if check_parity:
        par, steps, el, threads = opinion_parity(vh, run, g_oracle, x_init, args.hub_threshold)
        out["parity"] = par
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = {
                "value": E * steps / el, "unit": "edge-updates/s", "cores": threads,
                "kind": "port",
                "sample": "%d full steps (%.1f s) of the oracle's C restatement on the same "
                          "edges (the parity comparison's oracle run)" % (steps, el)}
        del g_oracle
    run.close()
    if rank == 0 and ws == 1 and args.secondary not in ("", "none"):
        out["secondary"] = run_secondaries(args)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_secondaries(args):
    """The other workloads, one process each (a failure of one leaves the
    headline line intact); each returns its own JSON line."""
    res = {}
    for name in [s.strip() for s in args.secondary.split(",") if s.strip()]:
        cmd = [sys.executable, os.path.abspath(__file__), "--workload", name, "--warmup", "3",
               "--seed", str(args.seed), "--cpu-seconds", str(args.cpu_seconds)]
        if name == "serve":
            cmd += ["--jobs", "1024", "--rates", "10,1000"]
        t0 = time.perf_counter()
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
            line = None
            for ln in reversed(r.stdout.splitlines()):
                if ln.strip().startswith("{"):
                    try:
                        line = json.loads(ln)
                        break
                    except ValueError:
                        pass
            if r.returncode != 0 or line is None:
                line = {"error": "rc %d: %s" % (r.returncode, (r.stderr or r.stdout)[-800:])}
        except subprocess.TimeoutExpired:
            line = {"error": "did not finish within 900 s"}
        line["wall_s"] = round(time.perf_counter() - t0, 1)
        res[name] = line
    return res


def run_batch(args):
    """Batched ensemble: 512 SIR instances (N log-uniform 1e3..1e5, out-degree
    5..30, beta 0.01..0.1, recovery 5..10, seed = instance index), 200 steps
    from the initial state, against the same instances stepped one at a time
    with the plain kernels (apply! per instance and step).

    The value is one call of `steps` steps from the initial state in the
    autotuner's form (mode 3), the autotuner having run before it (its time
    is reported apart; a graph form's capture stays inside the call).  Each
    form (graph replay, persistent grid launch, persistent cluster launch)
    is also timed from the initial state on a fresh copy of the ensemble,
    then once more over the next `steps` steps (the late epidemic), and
    every instance's final state of every form must be bit-identical to the
    plain path's."""
    import torch
    import vahana_gb300 as vh
    from vahana_gb300 import models
    vh.build()
    n_inst, steps = args.instances, args.batch_steps
    params = models.batch_params(n_inst)
    # warm-up on a small batch (graph capture machinery, autotuner)
    k = args.batch_warmup_instances
    if k > 0:
        w = models.Batch(*[p[:k] for p in params])
        w.step(steps, mode=3)
        w.close()

    def timed_step(b, mode):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.step(steps, mode=mode)
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    t0 = time.perf_counter()
    b = models.Batch(*params)
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    tune = b.tuning()  # the autotuner, on copies of the initial state
    t_tune = time.perf_counter() - t0
    t_auto = timed_step(b, 3)
    t0 = time.perf_counter()
    for i in range(n_inst):
        b.step_one(i, steps)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    plain = [b.states(i, 1) for i in range(n_inst)]

    def differing(bb):
        bad = 0
        for i in range(n_inst):
            sb, db = bb.states(i, 0)
            bad += int(not (np.array_equal(sb, plain[i][0]) and np.array_equal(db, plain[i][1])))
        return bad

    bad = {"auto": differing(b)}
    info = b.info()
    lanes = b.lanes()
    cluster = b.cluster()
    b.close()
    forms = {}
    for name, mode in (("graph_replay", 1), ("persistent_grid", 2), ("persistent_cluster", 4)):
        bf = models.Batch(*params)
        bf.tuning()
        t_first = timed_step(bf, mode)
        bad[name] = differing(bf)
        t_late = timed_step(bf, mode)
        bf.close()
        forms[name] = {"from_initial": n_inst * steps / t_first,
                       "late_epidemic": n_inst * steps / t_late}
    plain_rate = n_inst * steps / t_plain
    v = n_inst * steps / t_auto
    nbad = sum(bad.values())
    out = {"metric": "sim-steps/s", "value": v, "unit": "instance-steps/s", "n_gpus": 1,
           "steps": steps, "warmup": 1, "ms_per_step": 1e3 * t_auto / steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/i32",
           "data": "synthetic",
           "config": {"workload": "batched_sir_ensemble", "instances": n_inst,
                      "agents": info["agents"], "edges": info["edges"],
                      "from": "initial state",
                      "launch": {"tpb": info["tpb"], "agents_per_lane": lanes,
                                 "cluster": cluster},
                      "autotuner": tune},
           "build_seconds": t_build,
           "autotuner_seconds": t_tune,
           "first_call_with_autotuner": n_inst * steps / (t_tune + t_auto),
           "forms": forms,
           "plain_one_at_a_time": plain_rate,
           "speedup_vs_plain": v / plain_rate,
           "parity": {"instances": n_inst, "steps": steps,
                      "instances_differing_from_plain": bad, "pass": nbad == 0}}
    print(json.dumps(out), flush=True)


def serve_jobs(n_jobs, seed):
    """Job stream: model 50/50 SIR / opinion, N log-uniform in [1e3, 1e6],
    mean degree in [5, 30], 50..500 steps; SIR beta in [0.01, 0.1] and
    recovery 5..10; opinion eps 0.3 with the expected degree capped at
    min(1e4, N / 10)."""
    from vahana_gb300 import serve
    rng = np.random.default_rng(seed)
    specs = []
    for j in range(n_jobs):
        n = int(round(10 ** rng.uniform(3, 6)))
        steps = int(rng.integers(50, 501))
        if rng.random() < 0.5:
            specs.append(serve.sir_job(n, degree=int(rng.integers(5, 31)), steps=steps,
                                       seed=j + 1, beta=float(rng.uniform(0.01, 0.1)),
                                       recovery=int(rng.integers(5, 11))))
        else:
            specs.append(serve.opinion_job(n, mean_degree=float(rng.integers(5, 31)),
                                           steps=steps, seed=j + 1, eps=0.3,
                                           wmax=float(min(1e4, n / 10))))
    return specs


def run_serve(args):
    """Serving stream: args.jobs jobs arriving as a Poisson process at each
    rate of --rates, admitted by device footprint and stepped together; a
    sample of the jobs also runs one by one on the plain path (build, then
    apply! per step) for the throughput ratio and the per-job comparison."""
    import torch
    import vahana_gb300 as vh
    from vahana_gb300 import models, serve
    vh.build()
    specs = serve_jobs(args.jobs, args.seed)
    sample = list(range(min(args.plain_sample, len(specs))))
    for j in sample:
        specs[j].keep_state = 1
    total_steps = sum(s.steps for s in specs)
    # plain path, one job after the other, on the sample
    t0 = time.perf_counter()
    plain_states = {}
    for j in sample:
        s = specs[j]
        if s.model == serve.SIR:
            run = models.build_sir(n=s.n, degree=int(s.mean_degree), beta=s.beta,
                                   recovery=s.recovery, seed=s.seed)
            T = "Person"
        else:
            run = models.build_opinion(n=s.n, mean_degree=s.mean_degree, gamma=2.5, wmax=s.wmax,
                                       eps=s.eps, seed=s.seed,
                                       hub_threshold=models.OPINION_HUB_THRESHOLD)
            T = "Opinion"
        vh.finish_init(run.sim)
        for _ in range(s.steps):
            run.step()
        plain_states[j] = vh.read_agents(run.sim, T)[0]
        run.close()
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    plain_rate = sum(specs[j].steps for j in sample) / t_plain
    per_rate = []
    mismatched = 0
    rng = np.random.default_rng(args.seed + 1000)
    for rate in [float(r) for r in args.rates.split(",")]:
        arrivals = np.cumsum(rng.exponential(1.0 / rate, len(specs)))
        with serve.Server(budget_bytes=int(args.serve_budget_gb * (1 << 30))) as S:
            results = {}
            ids = []

            def feeder():
                t_start = time.perf_counter()
                for k, spec in enumerate(specs):
                    d = arrivals[k] - (time.perf_counter() - t_start)
                    if d > 0:
                        time.sleep(d)
                    ids.append(S.submit(spec))
            th = threading.Thread(target=feeder)
            th.start()
            deadline = time.perf_counter() + 1800
            while len(results) < len(specs):
                for r in S.poll():
                    results[r["id"]] = r
                if time.perf_counter() > deadline:
                    raise RuntimeError("serving stream did not finish within 30 minutes")
                time.sleep(0.002)
            th.join()
            stats = S.stats()
            lat = np.array([r["finish_s"] - r["arrival_s"] for r in results.values()])
            wait = np.array([r["admit_s"] - r["arrival_s"] for r in results.values()])
            t_first = min(r["arrival_s"] for r in results.values())
            t_last = max(r["finish_s"] for r in results.values())
            for j in sample:  # the sampled jobs' results equal their plain runs
                got = S.job_state(ids[j], specs[j])
                ref = plain_states[j]
                ok = (np.array_equal(got[0], ref["state"]) and np.array_equal(got[1], ref["days"])
                      if specs[j].model == serve.SIR
                      else np.array_equal(got.view(np.uint64), ref["x"].view(np.uint64)))
                mismatched += int(not ok)
        per_rate.append({"rate_jobs_per_s": rate, "p50_latency_s": float(np.percentile(lat, 50)),
                         "p99_latency_s": float(np.percentile(lat, 99)),
                         "p50_queue_wait_s": float(np.percentile(wait, 50)),
                         "sim_steps_per_s": total_steps / (t_last - t_first),
                         "makespan_s": t_last - t_first, "ticks": stats["ticks"]})
    best = max(per_rate, key=lambda r: r["sim_steps_per_s"])
    out = {"metric": "sim-steps/s", "value": best["sim_steps_per_s"], "unit": "job-steps/s",
           "n_gpus": 1, "steps": total_steps, "warmup": 0,
           "ms_per_step": 1e3 / best["sim_steps_per_s"], "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u8/i32+f64", "data": "synthetic",
           "config": {"workload": "serving_stream_sir_opinion", "jobs": len(specs),
                      "rates": [r["rate_jobs_per_s"] for r in per_rate],
                      "budget_gb": args.serve_budget_gb},
           "per_rate": per_rate,
           "plain_one_by_one": {"sim_steps_per_s": plain_rate, "sample_jobs": len(sample)},
           "speedup_vs_plain": best["sim_steps_per_s"] / plain_rate,
           "sample_jobs_differing_served_vs_alone": mismatched,
           "parity": {"sample_jobs": len(sample), "rates": len(per_rate),
                      "served_results_differing_from_alone": mismatched,
                      "pass": mismatched == 0}}
    print(json.dumps(out), flush=True)


def _timed_steps(step, stream, K, clk):
    """K steps between two events on the simulation's stream (no events
    inside the loop: at microseconds per step their own launch cost would be
    timed too); then, untimed, up to 100 steps with an event pair each for
    the distribution of single steps."""
    import torch
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    clk.start()
    time.sleep(0.3)
    start.record(stream)
    for k in range(K):
        step()
    end.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(min(K, 100))]
    for a, b in ev:
        a.record(stream)
        step()
        b.record(stream)
    torch.cuda.synchronize()
    per = sorted(a.elapsed_time(b) for a, b in ev)
    return start.elapsed_time(end), per, clocks


def run_model(args):
    """Config 0 (SIR, N = 10^5, out-degree 10, 100 steps) or config 2 (Life
    B3/S23 on a 4096 x 4096 periodic raster with 10^6 random walkers whose
    walker -> cell edges are rebuilt every step, 1000 steps): the same
    metric, edge-updates/s, for these parity workloads (the per-agent loop
    of apply! on each).  The oracle's C restatement runs every step the GPU
    ran, from the same initial state, and the final states (and, for Life,
    the rebuilt walker -> cell containers) must be bit-identical; that run,
    timed, is the CPU baseline."""
    import torch
    import vahana_gb300 as vh
    from vahana_gb300 import models
    from oracle import models as om
    vh.build()
    stream = torch.cuda.Stream()
    peak, kind = peaks()
    K = args.model_steps or (100 if args.workload == "sir" else 1000)
    if args.workload == "sir":
        N, deg = 100_000, 10
        run = models.build_sir(n=N, degree=deg, beta=0.05, recovery=7, seed=args.seed,
                               stream=stream.cuda_stream)
        frm, to, _ = models.staged_edges(run.sim, "Contact")
        st0, d0 = vh.read_agents(run.sim, "Person")[0].values()
        st0, d0 = st0.copy(), d0.copy()
        E = N * deg
        alg = 4 * E + 14 * N + 4
        cfg = {"workload": "sir_uniform_out_degree", "agents": N, "edges": E,
               "out_degree": deg, "beta": 0.05, "recovery": 7, "model_steps_reference": 100,
               "l2": "L2-resident (5.4 MB per step): latency bound"}
        kern = "k_sir"
    else:
        W = H = 4096
        nw = 1_000_000
        run = models.build_life(W, H, nw, 0.3, args.seed, stream=stream.cuda_stream)
        a0 = vh.read_agents(run.sim, "Cell")[0]["alive"].copy()
        wc = vh.read_agents(run.sim, "Walker")[0]
        x0, y0 = wc["x"].copy(), wc["y"].copy()
        E = 8 * W * H + nw
        alg = 2 * W * H + 16 * nw + 4 * (W * H + 1) + 4 * nw
        cfg = {"workload": "life_b3s23_raster_walkers", "raster": [W, H], "cells": W * H,
               "walkers": nw, "edges_per_step": E, "model_steps_reference": 1000,
               "l2": "inputs larger than L2 (121 MB per step)"}
        kern = "k_life2d + k_random_walk + walker edge rebuild"
    vh.finish_init(run.sim)
    vh.set_async(run.sim, True)
    for _ in range(args.warmup):
        run.step()
    vh.synchronize(run.sim)
    total_ms, per, clocks = _timed_steps(run.step, stream, K, Clocks(0))
    vh.synchronize(run.sim)
    done = args.warmup + K + len(per)  # model steps the GPU ran from the initial state
    mean_ms = total_ms / K
    out = {"metric": METRIC, "value": E * K / (total_ms * 1e-3), "unit": "edge-updates/s",
           "n_gpus": 1, "steps": K, "warmup": args.warmup, "ms_per_step": total_ms / K,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "u8/i32" if args.workload == "sir" else "bool/i32", "data": "synthetic",
           "config": cfg,
           "roofline": {"bound": "hbm", "achieved": alg / (mean_ms * 1e-3) / 1e9, "peak": peak,
                        "unit": "GB/s", "frac": alg / (mean_ms * 1e-3) / 1e9 / peak,
                        "peak_kind": kind, "traffic": None, "algorithmic_bytes_per_step": alg,
                        "kernel": kern, "step_ms_mean": mean_ms,
                        "single_step_ms_median": per[len(per) // 2]},
           "clocks": clocks, "gpu_launches_per_step": 1 if args.workload == "sir" else None}
    # oracle over the same `done` steps from the initial state (timed: the CPU baseline)
    t0 = time.perf_counter()
    if args.workload == "sir":
        s_ref, d_ref = om.run_sir(N, frm, to, st0, d0, 0.05, 7, args.seed, done, first_step=1)
        el = time.perf_counter() - t0
        cols = vh.read_agents(run.sim, "Person")[0]
        same = {"state": int((cols["state"] == s_ref).sum()),
                "days": int((cols["days"] == d_ref).sum())}
        passed = same["state"] == N and same["days"] == N
        out["parity"] = {"steps": done, "from": "initial state", "agents": N,
                         "agents_equal": same, "recovered": int((s_ref == 2).sum()),
                         "pass": bool(passed)}
    else:
        a_ref, x_ref, y_ref, rp_ref, src_ref = om.run_life_walkers(a0, x0, y0, W, H, args.seed,
                                                                  done)
        el = time.perf_counter() - t0
        a = vh.read_agents(run.sim, "Cell")[0]["alive"].astype(np.uint8)
        wk = vh.read_agents(run.sim, "Walker")[0]
        rp, frm_c, _ = vh.read_edges(run.sim, "OnCell", "Cell")
        src_c = frm_c & np.uint64((1 << 36) - 1)
        same = {"cells": int((a == a_ref).sum()),
                "walkers": int(((wk["x"] == x_ref) & (wk["y"] == y_ref)).sum()),
                "oncell_row_ptr_equal": bool(np.array_equal(rp, rp_ref)),
                "oncell_sources_equal": bool(np.array_equal(src_c, src_ref))}
        passed = (same["cells"] == W * H and same["walkers"] == nw
                  and same["oncell_row_ptr_equal"] and same["oncell_sources_equal"])
        out["parity"] = {"steps": done, "from": "initial state", "cells_and_walkers_equal": same,
                         "alive_cells": int(a_ref.sum()), "pass": bool(passed)}
    if not args.no_cpu_baseline and args.workload == "sir":
        # the parity run lasts a few hundredths of a second: time the
        # oracle's steps again (the in-edge lists built once, outside the
        # clock), whole runs from the initial state, for a quarter of
        # --cpu-seconds
        g = om.build_inedges(N, frm, to)
        runs, t0 = 0, time.perf_counter()
        while runs == 0 or time.perf_counter() - t0 < args.cpu_seconds / 4:
            s, d = np.ascontiguousarray(st0, np.uint8), np.ascontiguousarray(d0, np.int32)
            for t in range(done):
                s, d = om.sir_step(g, s, d, 0.05, 7, args.seed, 1 + t)
            runs += 1
        el_cpu = time.perf_counter() - t0
        same_again = bool(np.array_equal(s, s_ref) and np.array_equal(d, d_ref))
        out["cpu_baseline"] = {"value": E * done * runs / el_cpu, "unit": "edge-updates/s",
                               "cores": om.threads(), "kind": "port",
                               "sample": "%d runs of the parity run's %d steps (%.2f s) of the "
                                         "oracle's C restatement" % (runs, done, el_cpu),
                               "runs_equal_parity_run": same_again}
    elif not args.no_cpu_baseline:
        out["cpu_baseline"] = {"value": E * done / el, "unit": "edge-updates/s",
                               "cores": om.threads(), "kind": "port",
                               "sample": "%d steps (%.1f s) of the oracle's C restatement "
                                         "(the parity run)" % (done, el)}
    run.close()
    print(json.dumps(out), flush=True)


def run_rates(args):
    """Arithmetic throughput of this GPU (vg_selftest_rate): binary64 add,
    multiply and fused multiply-add, the gather kernel's integer-pipe
    product and a 32-bit integer multiply-add, with every lane of a warp
    active, and the binary64 add with part of each warp's lanes active.  The
    last figure bounds the gather kernel of the opinion workload, which
    issues two binary64 additions per edge: 2 E / (add rate) per step."""
    import ctypes as C
    import torch  # noqa: F401  (CUDA context in the same process as the sampler)
    import vahana_gb300 as vh
    from vahana_gb300._lib import check, lib
    vh.build()
    names = {0: "dadd", 1: "dmul", 2: "dfma", 3: "emu_mul_grid", 4: "int32_mad_or"}
    blocks = 152 * 8
    ms, ops = C.c_double(), C.c_double()
    runs = [(m, 32) for m in range(5)] + [(0, 16), (0, 8), (0, 1)]
    clk = Clocks(0)
    clk.start()
    time.sleep(0.3)
    res = []
    for mode, lanes in runs:
        iters = 1 << 14 if mode in (0, 1, 2) else 1 << 12
        check(lib().vg_selftest_rate(mode, blocks, iters, lanes, C.byref(ms), C.byref(ops)))
        res.append({"op": names[mode], "active_lanes": lanes, "ms": ms.value,
                    "lane_ops_per_s": ops.value / (ms.value * 1e-3),
                    "warp_instr_per_s": ops.value / lanes / (ms.value * 1e-3)})
    clocks = clk.stop()
    mhz = clocks.get("sm_mhz") or 2070.0
    for r in res:
        r["lane_ops_per_sm_per_clock"] = r["lane_ops_per_s"] / (152 * mhz * 1e6)
    dadd = res[0]["lane_ops_per_s"]
    E = 200_000_000
    out = {"metric": "binary64 add/s", "value": dadd, "unit": "lane-ops/s", "n_gpus": 1,
           "steps": len(runs), "warmup": 1, "ms_per_step": res[0]["ms"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": {"workload": "arithmetic_throughput",
                                           "blocks": blocks, "threads_per_block": 256,
                                           "chains_per_thread": 8},
           "rates": res, "clocks": clocks,
           "opinion_step_fp64_floor_ms": 2 * E / dadd * 1e3,
           "opinion_step_fp64_floor_note": "two binary64 additions per edge, E = 2e8"}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.workload == "fp64":
        run_rates(args)
        return
    if args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload in ("sir", "life"):
        run_model(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
