"""Multi-rank path on CPU: two gloo ranks shard a batch, solve their shards with the
CPU oracle, and reduce; the totals equal a single-process run."""
import os
import sys

import pytest

from conftest import ROOT


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    import oracle as og
    from relaibilitygpu_gb300 import graphs, replicas
    dist.init_process_group("gloo", rank=rank, world_size=world)
    gs = [graphs.complete(9, p_range=(0.8, 0.99), seed=s) for s in range(50)]
    b, e = replicas.shard(len(gs), rank, world)
    nodes = leaves = 0
    for g in gs[b:e]:
        r = og.run(g, 0, 8, bucket_shift=0, n_buckets=64, target_width=1e-6)
        nodes += r.nodes
        leaves += r.leaves
    tot = replicas.reduce_totals({"nodes": nodes, "leaves": leaves, "instances": e - b, "rank_max": rank})
    q.put((rank, tot))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_covers_everything():
    from relaibilitygpu_gb300 import replicas
    for n in (0, 1, 7, 100):
        for world in (1, 2, 3, 8):
            spans = [replicas.shard(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1


def test_two_gloo_ranks_match_single_process():
    import multiprocessing as mp
    import socket
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as og
    from relaibilitygpu_gb300 import graphs
    og.lib()
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    gs = [graphs.complete(9, p_range=(0.8, 0.99), seed=s) for s in range(50)]
    nodes = sum(og.run(g, 0, 8, bucket_shift=0, n_buckets=64, target_width=1e-6).nodes for g in gs)
    for r in (0, 1):
        assert out[r]["nodes"] == nodes
        assert out[r]["instances"] == 50
        assert out[r]["rank_max"] == 1
