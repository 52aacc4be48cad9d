"""Multi-rank helpers: independent replicas, no collective on the data path.

Instances of a batch are independent, so N ranks (one GPU each) either solve
disjoint shards of one batch (strong scaling) or one batch each (weak
scaling).  The only communication is one reduction of the per-rank totals at
the end: subproblem counts are summed, times take the maximum (the slowest
rank sets the job's time), and exact mass sums are added in integer space.
"""
from __future__ import annotations

from typing import Dict, Tuple


def shard(n: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous [begin, end) slice of n instances for this rank; sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def reduce_totals(local: Dict[str, float], group=None) -> Dict[str, float]:
    """Combine per-rank totals: '*_max' keys take the maximum, every other key is summed."""
    import torch
    import torch.distributed as dist
    keys = sorted(local)
    sums = torch.tensor([float(local[k]) for k in keys if not k.endswith("_max")], dtype=torch.float64)
    maxs = torch.tensor([float(local[k]) for k in keys if k.endswith("_max")], dtype=torch.float64)
    if dist.is_available() and dist.is_initialized():
        backend = dist.get_backend(group)
        dev = "cuda" if backend == "nccl" else "cpu"
        sums, maxs = sums.to(dev), maxs.to(dev)
        if sums.numel():
            dist.all_reduce(sums, op=dist.ReduceOp.SUM, group=group)
        if maxs.numel():
            dist.all_reduce(maxs, op=dist.ReduceOp.MAX, group=group)
        sums, maxs = sums.cpu(), maxs.cpu()
    out, i, j = {}, 0, 0
    for k in keys:
        if k.endswith("_max"):
            out[k] = float(maxs[j]); j += 1
        else:
            out[k] = float(sums[i]); i += 1
    return out
