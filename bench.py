"""Benchmark of the GB300 reliability engine (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Workloads (all synthetic, seeded; numpy PCG64):
  k15batch (default) -- the metric's configuration: K15 (N=15, E=105), src 0,
      dst 14, edge p ~ U[0.9, 0.99] FP64, run in plain max-mass order until the
      ESP width (ESP + queued mass) is <= 1e-6.  One instance needs only ~20-60
      subproblems, so a step solves a batch of 4096 such instances (seeds
      0..4095) in one launch; single-instance time-to-bound is reported beside it.
  k10 -- K10 (N=10, E=45), p ~ U[0.5, 0.95], exhaustive (one solve per step).
  k15p05, k25p05 -- the reference's own published K15 / K25 p=0.5 runs
      (breadth-first waves, 77,410,924-slot wave buffers, eps 1e-15).
  rgg200 -- random geometric graph N=200, E=600 (unit square, terminals the
      farthest pair), p ~ U[0.9, 0.99]: the whole-GPU bucketed max-mass queue
      aiming at ESP width <= 1e-5, stopped at a budget of 20M subproblems per
      step (the bound is far beyond one GPU's queue memory; the line reports
      the R <= true <= R + ESP bracket reached).

`value` is subproblems (popped nodes, dead ends included) per second of
device time: the engine's CUDA events on its own stream around the kernels,
summed over ranks and divided by the slowest rank.  `e2e` is the same metric
with wall-clock time around the public C call (graph tables host->device,
results device->host).  L2 is flushed (a 512 MB write) before every step.

--impl reference times the reference algorithm on the host cores: the CPU
port in oracle/ (the reference's own seq/seq.cpp needs the reference tree,
which the GPU host does not have), one instance per thread, every host
thread.  Multi-GPU runs are independent replicas: each rank solves its own
copy of the workload; no collective on the data path.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "time to ESP<=1e-6 on K15, learned vs plain order (1 GB300); subproblems/sec"
UNIT = "subproblems/sec"
BATCH = 4096


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def workload(name: str):
    import relaibilitygpu_gb300 as nr
    if name == "k15batch":
        gs = [nr.complete(15, p_range=(0.9, 0.99), seed=s) for s in range(BATCH)]
        return dict(kind="batch", graphs=gs, srcs=[0] * BATCH, dsts=[14] * BATCH, capacity=0,
                    opts=dict(target_width=1e-6, bucket_shift=2, n_buckets=256),
                    oracle=dict(bucket_shift=2, n_buckets=256, target_width=1e-6),
                    name=f"K15 (N=15, E=105) src=0 dst=14 p~U[0.9,0.99] seeds 0..{BATCH - 1}, "
                         f"max-mass order to ESP width<=1e-6, {BATCH} instances per step")
    if name in ("k15p05", "k25p05"):
        n = 15 if name == "k15p05" else 25
        g = nr.complete(n, p=0.5)
        return dict(kind="single", graphs=[g], srcs=[0], dsts=[n - 1], capacity=77410924,
                    opts=dict(eps=1e-15), oracle=dict(eps=1e-15, max_nodes=20_000_000),
                    name=f"K{n} p=0.5 (COMP{n}-05.txt) src=0 dst={n - 1}, breadth-first waves, queue capacity "
                         f"77,410,924 per wave buffer, truncation eps 1e-15 (the reference's own published run)")
    if name == "rgg200":
        g = nr.rgg(200, 600, p_range=(0.9, 0.99), seed=7)
        opts = dict(target_width=1e-5, order="maxmass", bucket_shift=2, n_buckets=255, max_nodes=20_000_000,
                    timeout_ms=120000.0)
        return dict(kind="single", graphs=[g], srcs=[g.src], dsts=[g.dst], capacity=1 << 28, opts=opts,
                    oracle=dict(target_width=1e-5, bucket_shift=2, n_buckets=255, max_nodes=1_000_000),
                    name=f"RGG N=200 E={g.n_edges} (unit square, seed 7) src={g.src} dst={g.dst} (farthest pair) "
                         f"p~U[0.9,0.99], bucketed max-mass order (4 buckets per octave) toward ESP width <=1e-5, "
                         f"20M-subproblem budget per step, 2^28-slot arena")
    if name == "k10":
        g = nr.complete(10, p_range=(0.5, 0.95), seed=2)
        return dict(kind="single", graphs=[g], srcs=[0], dsts=[9], capacity=1 << 22, opts=dict(eps=0.0),
                    oracle=dict(), name="K10 (N=10, E=45) src=0 dst=9 p~U[0.5,0.95] seed 2, exhaustive")
    raise SystemExit(f"unknown workload {name}")


# DRAM bytes (read + write) of one launch of the dominant kernel, from one ncu capture of the same
# workload (the launch summaries are kept under profiles/).
TRAFFIC = {"k15batch": 4.194e6, "k10": 136.8e6}


def item_bytes(n_edges: int) -> int:
    """Algorithmic bytes of one queued subproblem: packed 2-bit mask words + FP64 mass."""
    return 4 * max(1, (2 * n_edges + 31) // 32) + 8


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while timing."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
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
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU port (oracle/): instances in parallel, one per host thread
# ---------------------------------------------------------------------------
def cpu_solve_all(w, threads: int, reps: int = 1, _cache={}):
    import oracle as og
    og.lib()
    t0 = time.perf_counter()
    nodes = 0
    if w["kind"] == "single":
        for _ in range(reps):
            for g, s, d in zip(w["graphs"], w["srcs"], w["dsts"]):
                nodes += og.run(g, s, d, threads=threads, **w["oracle"]).nodes
    else:
        key = id(w)
        if key not in _cache:
            _cache[key] = og.BatchArgs(w["graphs"], w["srcs"], w["dsts"])
        t0 = time.perf_counter()
        for _ in range(reps):
            res = og.run_batch(_cache[key], threads=threads, **w["oracle"])
            nodes += sum(res[i].nodes for i in range(len(w["graphs"])))
    secs = time.perf_counter() - t0
    return nodes, secs, threads


def cpu_baseline(w, threads: int):
    # bounded sample: repeat the whole workload until about 2 s of host time has passed
    nodes, secs, used = cpu_solve_all(w, threads, 1)
    reps = max(1, min(50, int(2.0 / max(secs, 1e-3))))
    if reps > 1:
        nodes, secs, used = cpu_solve_all(w, threads, reps)
    return {"value": nodes / secs, "unit": UNIT, "cores": used, "kind": "port",
            "sample": f"{reps} x the full workload ({len(w['graphs'])} instance(s)), oracle/pathdecomp.c, "
                      f"same schedule and stop rule, {used} host threads"}


def stored_schedule(w):
    """The oracle schedule of the autotuner's choice on GB300 for a batch workload: breadth-first
    waves (one bucket) to the workload's target width."""
    w["oracle"] = dict(bucket_shift=-1, n_buckets=1, target_width=w["opts"]["target_width"])


def stored_tuning(w):
    """A batch workload with the autotuner's choice on GB300 (breadth-first waves, 2 warps a block,
    64 pages a warp): the options of --no-autotune, and the oracle schedule they correspond to."""
    import relaibilitygpu_gb300 as nr
    tuned = dict(nr.options_dict(nr.make_options(**w["opts"])), bucket_shift=-1, n_buckets=64,
                 warps_per_block=2, pages_per_warp=64)
    stored_schedule(w)
    w["opts"] = tuned
    return tuned


def run_reference(args, rank, world):
    if rank != 0:
        return
    w = workload(args.workload)
    if w["kind"] == "batch":
        stored_schedule(w)                # the schedule our arm runs (and its CPU baseline times)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_solve_all(w, threads, 1)
    nodes, secs = 0, 0.0
    for _ in range(args.steps):
        n, s, _ = cpu_solve_all(w, threads, 1)
        nodes += n
        secs += s
    value = nodes / secs
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": w["name"], "parallelism": f"{threads} host threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"full workload per step, oracle/pathdecomp.c, {threads} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="k15batch")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true",
                    help="k15batch: skip the plain / learned / breadth-first order comparison")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batch workloads: use the stored tuned settings instead of running nr_autotune")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)

    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch
    import relaibilitygpu_gb300 as nr
    from relaibilitygpu_gb300 import build as nb
    nb.build()
    torch.cuda.set_device(local)
    w = workload(args.workload)
    ctx = nr.Context(local)
    batch = nr.Batch(w["graphs"], w["srcs"], w["dsts"])
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    tuned = None
    if w["kind"] == "batch" and args.no_autotune:
        tuned = stored_tuning(w)
    elif w["kind"] == "batch":
        # autotuner (nr_autotune): bucket resolution, pages per warp, warps per block
        tuned, tuned_ms = nr.autotune(ctx, batch, capacity=w["capacity"], **w["opts"])
        w["opts"] = tuned
        w["oracle"] = dict(bucket_shift=tuned["bucket_shift"],
                           n_buckets=tuned["n_buckets"] if tuned["bucket_shift"] >= 0 else 1,
                           target_width=tuned["target_width"])

    def call():
        if w["kind"] == "batch":
            return ctx.run_batch(batch, capacity=w["capacity"], raw=True, **w["opts"])
        return [ctx.reliability(w["graphs"][0], w["srcs"][0], w["dsts"][0], capacity=w["capacity"],
                                **w["opts"])._raw]

    for _ in range(max(3, args.warmup)):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        call()
    sampler = ClockSampler(local)
    sampler.start()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    dev_ms, wall_s, nodes, abytes = 0.0, 0.0, 0, 0
    per_step = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = call()
        wall_s += time.perf_counter() - t0
        ms = res[0].ms
        n_step = sum(r.nodes for r in res)
        b_step = sum((r.nodes + max(0, r.nodes - 1 + r.queued)) * item_bytes(r.n_edges) for r in res)
        dev_ms += ms
        nodes += n_step
        abytes += b_step
        per_step.append((ms, n_step, b_step))
    torch.cuda.synchronize()
    # e2e through the asynchronous API: two batches in flight, so the host builds one step's
    # tables while the GPU runs the step before.  Every step still uploads its inputs from
    # pinned host memory and reads its results back; the L2 flush of each step runs on its
    # own stream and the step's upload is ordered after it.
    e2e_pipe = None
    if w["kind"] == "batch":
        batches = [batch, nr.Batch(w["graphs"], w["srcs"], w["dsts"])]
        fs = torch.cuda.Stream(device=f"cuda:{local}")
        # 192 MB (1.5x the 129 MB L2) evicts the previous steps' lines; a bigger write would only
        # take HBM time from the step running beside it.  The write is a cudaMemsetAsync on the
        # flush stream, issued through the CUDA runtime that libnr.so links (a few microseconds of
        # host time, where a torch fill under a stream context costs tens)
        import ctypes
        cudart = ctypes.CDLL("libcudart.so.13")
        cudart.cudaMemsetAsync.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p]
        cudart.cudaMemsetAsync.restype = ctypes.c_int
        flush_args = (ctypes.c_void_p(flush.data_ptr()), 1, ctypes.c_size_t(192 * 1024 * 1024),
                      ctypes.c_void_p(fs.cuda_stream))

        pipe_opts = nr.make_options(**w["opts"])

        def pipelined(steps):
            pending = None
            for k in range(steps):
                if cudart.cudaMemsetAsync(*flush_args) != 0:
                    raise RuntimeError("cudaMemsetAsync (L2 flush) failed")
                tk = ctx.submit(batches[k % 2], capacity=w["capacity"], after_stream=fs.cuda_stream, options=pipe_opts)
                if pending is not None:
                    ctx.wait(pending)
                pending = tk
            ctx.wait(pending)

        pipelined(max(3, args.warmup))
        torch.cuda.synchronize()
        # a pipelined call stream is measured in its steady state: at least 50 steps, so the
        # filling and draining of the two-batch pipeline are a small part of the time
        e2e_steps = max(args.steps, 50)
        t0 = time.perf_counter()
        pipelined(e2e_steps)
        t_pipe = time.perf_counter() - t0
        torch.cuda.synchronize()
        # every step solves the same instances: count the subproblems of each batch's last step
        per_batch = [sum(bb.res[i].nodes for i in range(bb.n)) for bb in batches]
        n_pipe = sum(per_batch[k % 2] for k in range(e2e_steps))
        e2e_pipe = (n_pipe, t_pipe)
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    r0 = res[0]
    # the batch's result array is reused by the comparison runs below: keep the timed run's figures
    grid0, block0 = int(r0.grid_blocks), int(r0.block_threads)
    h2d = sum(r.h2d_bytes for r in res)
    d2h = sum(r.d2h_bytes for r in res)
    stats = {"R": r0.R, "R_plus_esp": r0.R_plus_esp, "esp": r0.esp, "paths": int(r0.paths), "nodes": int(r0.nodes),
             "iterations": int(r0.iterations), "queued": int(r0.queued), "spilled": int(r0.spilled),
             "stop": {0: "queue empty", 1: "target width met", 3: "node budget"}.get(int(r0.stop), int(r0.stop)),
             "engine": nr.engine.ENGINES.get(r0.engine, r0.engine),
             "kernel": nr.engine.KERNELS.get(r0.kernel, r0.kernel), "nodes_per_step": nodes // args.steps}

    # single-instance time-to-bound (latency): plain max-mass order vs the learned order
    ttb = None
    if args.workload == "k15batch" and not args.no_compare:
        from relaibilitygpu_gb300 import learned as LR

        # the order comparison runs at one bucket resolution (one bucket per factor of two), since
        # with a single bucket (breadth-first waves) there is nothing for a priority to reorder
        cmp_opts = {k: v for k, v in w["opts"].items() if k not in ("order", "bucket_shift", "n_buckets")}
        cmp_opts.update(bucket_shift=0, n_buckets=64)

        def latency(order, **kw):
            tk, tb, nd = [], [], []
            for s in range(16):
                r = ctx.reliability(w["graphs"][s], 0, 14, order=order, **{**cmp_opts, **kw})
                tk.append(r.ms)
                tb.append(r.time_to_bound_ms)
                nd.append(r.nodes)
            return {"kernel_us_median": 1e3 * statistics.median(tk),
                    "in_kernel_us_median": 1e3 * statistics.median(tb),
                    "nodes_mean": statistics.mean(nd)}

        def batch_run(order):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            rr = ctx.run_batch(batch, capacity=w["capacity"], raw=True, order=order, **cmp_opts)
            nn = sum(rr[i].nodes for i in range(len(w["graphs"])))
            return {"ms": rr[0].ms, "nodes": nn, "subproblems_per_sec": nn / (rr[0].ms / 1e3)}

        def per_graph_launches():
            # the same 4096 instances one call (one launch) each, with the batch's tuned settings
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            nn, dev = 0, 0.0
            for g, s_, d_ in zip(w["graphs"], w["srcs"], w["dsts"]):
                r = ctx.reliability(g, s_, d_, capacity=w["capacity"], **w["opts"])
                nn += r.nodes
                dev += r.ms
            wall = time.perf_counter() - t0
            return {"launches": len(w["graphs"]), "wall_ms": 1e3 * wall, "device_ms_sum": dev,
                    "subproblems_per_sec_wall": nn / wall, "subproblems_per_sec_device": nn / (dev / 1e3)}

        try:
            ttb = {"plain": latency("maxmass"), "learned": None, "instances": 16,
                   "breadth_first": latency("maxmass", bucket_shift=-1),
                   "fork_branching": latency("maxmass", branching="fork"),
                   "plain_batch": batch_run("maxmass"),
                   "per_graph_launches": per_graph_launches()}
        except Exception as exc:                     # keep the bench line; report the failure
            ttb = {"plain": f"failed: {exc}", "learned": None, "instances": 16}
        if os.path.exists(LR.DEFAULT_MODEL) and isinstance(ttb["plain"], dict):
            LR.set_model(ctx, LR.load())
            ttb["learned"] = latency("learned")
            ttb["learned_batch"] = batch_run("learned")
        elif not os.path.exists(LR.DEFAULT_MODEL):
            ttb["learned"] = "no model file (python -m relaibilitygpu_gb300.learned train)"

    t_dev = dev_ms / 1e3
    # replicas: units add up over ranks, the slowest rank sets the time (no data-path collective)
    from relaibilitygpu_gb300 import replicas
    red = {"nodes": float(nodes), "t_dev_max": t_dev, "wall_max": wall_s}
    if e2e_pipe is not None:
        red.update(pipe_nodes=float(e2e_pipe[0]), pipe_wall_max=e2e_pipe[1])
    tot = replicas.reduce_totals(red)
    tot_nodes, t_dev, wall_s = tot["nodes"], tot["t_dev_max"], tot["wall_max"]
    if rank != 0:
        ctx.close()
        if dist is not None:
            dist.destroy_process_group()
        return
    peak, peak_kind = peaks()
    achieved = statistics.mean(b / (ms / 1e3) / 1e9 for ms, _, b in per_step)
    line = {
        "metric": METRIC, "value": tot_nodes / t_dev, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": w["name"], "l2": "flushed (512 MB write) before every step",
                   "parallelism": f"replicas x{world}", "engine": stats["engine"], "kernel": stats["kernel"],
                   "grid": grid0, "block": block0,
                   "autotuned": None if tuned is None else {k: tuned[k] for k in
                                                             ("bucket_shift", "n_buckets", "warps_per_block",
                                                              "pages_per_warp")}},
        "result": stats,
        "time_to_bound": ttb,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": TRAFFIC.get(args.workload),
                     "note": f"achieved = algorithmic bytes (4W+8 per queued subproblem, written once and "
                             f"read once) / kernel time; peak {peak_kind} copy bandwidth; traffic = DRAM "
                             f"bytes read + written per launch in one ncu capture (profiles/), the queue "
                             f"itself stays in L2"},
        "e2e": ({"value": tot["pipe_nodes"] / tot["pipe_wall_max"], "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                 "d2h_bytes_per_step": int(d2h),
                 "api": "nr_batch_submit / nr_batch_wait, two batches in flight; L2 flushed (192 MB write) before "
                        "every step's upload, on its own stream, the upload ordered after it",
                 "steps": e2e_steps, "one_call_at_a_time": tot_nodes / wall_s}
                if e2e_pipe is not None else
                {"value": tot_nodes / wall_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                 "d2h_bytes_per_step": int(d2h), "api": "one synchronous call per step"}),
        "gpu_launches": args.steps * (len({(r.n_nodes, r.mask_words) for r in res}) if w["kind"] == "batch" else 1),
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, os.cpu_count() or 1)
    print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
