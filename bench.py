"""Benchmark of the GB300 reliability engine (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

A step is one solve of the workload through the C ABI.  `value` is
subproblems (popped nodes) per second of device time, summed over ranks and
divided by the slowest rank; the device time of each step is the kernel's
CUDA-event time on the engine's own stream.  `e2e` is the same metric with
wall-clock time around the public call (graph tables host->device, results
device->host).  L2 is flushed (a 512 MB write) before every timed step.

--impl reference times the reference algorithm's CPU implementation on the
host cores: the CPU port in oracle/ (the reference's own seq.cpp cannot be
built on the GPU host, which has no reference tree), with every host thread.
Multi-GPU runs are independent replicas (the decomposition shards, but each
rank solves its own copy of the workload; no collective on the data path).
"""
from __future__ import annotations

import argparse
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
    if name == "k10":
        g = nr.complete(10, p_range=(0.5, 0.95), seed=2)
        return dict(name="K10 (N=10, E=45) src=0 dst=9 p~U[0.5,0.95] seed 2, exhaustive",
                    graph=g, src=0, dst=9, capacity=1 << 22, opts=dict(eps=0.0))
    raise SystemExit(f"unknown workload {name}")


def algorithmic_bytes(n_edges: int, nodes: int, pushes: int) -> int:
    """Each queued subproblem is written once and read once: S = 4*W + 8 bytes
    (packed 2-bit mask words + FP64 mass)."""
    W = max(1, (2 * n_edges + 31) // 32)
    return (nodes + pushes) * (4 * W + 8)


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


def cpu_port(w, threads: int, sample_note: str):
    import oracle as og
    r = og.run(w["graph"], w["src"], w["dst"], threads=threads, eps=w["opts"].get("eps", 0.0))
    return {"value": r.nodes / r.seconds, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": sample_note, "nodes": r.nodes, "seconds": r.seconds}


def run_reference(args, rank, world):
    if rank != 0:
        return
    import oracle as og
    og.lib()
    w = workload(args.workload)
    threads = os.cpu_count() or 1
    vals = []
    for i in range(args.warmup + args.steps):
        r = og.run(w["graph"], w["src"], w["dst"], threads=threads, eps=w["opts"].get("eps", 0.0))
        if i >= args.warmup:
            vals.append((r.nodes, r.seconds))
    nodes = sum(v[0] for v in vals)
    secs = sum(v[1] for v in vals)
    value = nodes / secs
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": w["name"], "parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"full workload per step, oracle/pathdecomp.c waves schedule, {threads} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="k10")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        import torch
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
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def step():
        flush.fill_(1.0)
        torch.cuda.synchronize()
        return ctx.reliability(w["graph"], w["src"], w["dst"], capacity=w["capacity"], **w["opts"])

    for _ in range(max(3, args.warmup)):
        step()
    sampler = ClockSampler(local)
    sampler.start()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    dev_ms, wall_s, nodes, pushes = 0.0, 0.0, 0, 0
    results = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = ctx.reliability(w["graph"], w["src"], w["dst"], capacity=w["capacity"], **w["opts"])
        wall_s += time.perf_counter() - t0
        dev_ms += r.ms
        nodes += r.nodes
        pushes += r.nodes - 1 - r.truncated * 0   # every pop but the root was a push
        results.append(r)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()

    t_dev = dev_ms / 1e3
    if dist is not None:
        t = torch.tensor([t_dev, wall_s, float(nodes)], dtype=torch.float64, device=f"cuda:{local}")
        tmax = t.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        tsum = t.clone()
        dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
        t_dev, wall_s, tot_nodes = float(tmax[0]), float(tmax[1]), float(tsum[2])
    else:
        tot_nodes = float(nodes)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    r0 = results[0]
    peak, peak_kind = peaks()
    bytes_per_step = algorithmic_bytes(r0.n_edges, r0.nodes, r0.nodes - 1)
    achieved = bytes_per_step / (r0.ms / 1e3) / 1e9 if r0.ms > 0 else 0.0
    ach = [algorithmic_bytes(r.n_edges, r.nodes, r.nodes - 1) / (r.ms / 1e3) / 1e9 for r in results]
    achieved = statistics.mean(ach)
    line = {
        "metric": METRIC, "value": tot_nodes / t_dev, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": w["name"], "l2": "flushed (512 MB write) before every step",
                   "parallelism": f"replicas x{world}", "engine": r0.engine, "grid": r0.grid_blocks,
                   "block": r0.block_threads},
        "result": {"R": r0.R, "esp": r0.esp, "paths": r0.paths, "nodes": r0.nodes, "iterations": r0.iterations,
                   "max_queue_items": r0.max_queue_items},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "note": f"algorithmic bytes (4W+8 per queued subproblem, read+write) / kernel time; "
                             f"peak {peak_kind}"},
        "e2e": {"value": tot_nodes / wall_s, "unit": UNIT, "h2d_bytes_per_step": r0.h2d_bytes,
                "d2h_bytes_per_step": r0.d2h_bytes},
        "gpu_launches": args.steps,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        line["cpu_baseline"] = cpu_port(w, threads, f"one full solve of the workload, {threads} threads")
    print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
