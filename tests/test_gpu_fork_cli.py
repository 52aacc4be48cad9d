"""Fork branching (the reference's FORK_BEST_EDGE mode, workingPad/main.cu:303-430 with
:550-565) on every engine against the oracle, and the drop-in `network_reliability` program."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import rel_close

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "relaibilitygpu_gb300", "network_reliability")


@pytest.fixture(scope="module")
def ctx(engine_lib):
    c = engine_lib.Context(0)
    yield c
    c.close()


def check(r, o):
    assert (r.nodes, r.leaves, r.dead_ends, r.truncated, r.spilled, r.paths) == \
        (o.nodes, o.leaves, o.dead, o.truncated, o.spilled, o.paths)
    assert r.R == o.R, (r.R, o.R)
    assert r.esp == o.esp, (r.esp, o.esp)


def test_fork_whole_gpu_waves_exhaustive(ctx, oracle, load_golden_graph):
    """Exhaustive breadth-first waves (the reference's own schedule): same waves, counts, R."""
    from relaibilitygpu_gb300 import graphs
    cases = [(load_golden_graph("COMP8"), 0, 7), (load_golden_graph("COMP9"), 0, 8),
             (graphs.grid(4, 4, p=0.9), 0, 15), (graphs.gnm(18, 32, p_range=(0.5, 0.95), seed=5), None, None)]
    for g, s, t in cases:
        s = g.src if s is None else s
        t = g.dst if t is None else t
        o = oracle.run(g, s, t, branching="fork", threads=4)
        r = ctx.reliability(g, s, t, capacity=1 << 22, branching="fork")
        assert r.engine == "grid"
        check(r, o)
        assert (r.iterations, r.max_queue_items) == (o.waves, o.max_wave)
        assert rel_close(r.R, oracle.brute(g, s, t), 1e-12) if g.n_edges <= 30 else True


@pytest.mark.parametrize("shift", [-1, 0, 2])
def test_fork_warp_engine_truncated(ctx, oracle, shift):
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(n, p_range=(0.85, 0.99), seed=70 + n) for n in (6, 9, 12, 15, 20, 27, 32)]
    nb = 64 if shift >= 0 else 1
    res = ctx.reliability_batch(gs, [0] * len(gs), [g.n_nodes - 1 for g in gs], capacity=1 << 16,
                                target_width=1e-7, bucket_shift=shift, n_buckets=64, branching="fork")
    for g, r in zip(gs, res):
        o = oracle.run(g, 0, g.n_nodes - 1, branching="fork", target_width=1e-7, bucket_shift=shift,
                       n_buckets=nb)
        assert r.engine == "warp"
        check(r, o)
        assert (r.iterations, r.max_queue_items, r.queued, r.stop) == (o.waves, o.max_wave, o.queued, o.status)


def test_fork_wide_engines(ctx, oracle):
    from relaibilitygpu_gb300 import graphs
    g = graphs.rgg(60, 150, p_range=(0.9, 0.99), seed=11)
    for target, kw in ((1e-4, dict(bucket_shift=-1)), (1e-6, dict(order="maxmass", bucket_shift=2, n_buckets=255))):
        okw = dict(bucket_shift=kw["bucket_shift"], n_buckets=kw.get("n_buckets", 1))
        o = oracle.run(g, g.src, g.dst, branching="fork", target_width=target, threads=4, **okw)
        r = ctx.reliability(g, g.src, g.dst, capacity=1 << 22, target_width=target, branching="fork", **kw)
        assert r.engine == "grid"
        check(r, o)
        assert (r.iterations, r.max_queue_items, r.queued) == (o.waves, o.max_wave, o.queued)
    k40 = graphs.complete(40, p_range=(0.9, 0.99), seed=1)
    o = oracle.run(k40, 0, 39, branching="fork", target_width=1e-9)
    r = ctx.reliability(k40, 0, 39, capacity=1 << 20, target_width=1e-9, branching="fork", bucket_shift=-1)
    check(r, o)


def test_fork_rejects_learned_order(ctx, engine_lib):
    from relaibilitygpu_gb300 import graphs
    with pytest.raises(engine_lib.NrError):
        ctx.reliability(graphs.complete(6, p=0.5), 0, 5, order="learned", branching="fork")


def parse_block(text):
    def num(pat):
        m = re.search(pat, text)
        assert m, (pat, text)
        return m.group(1)
    return {"R": float(num(r"Reliability:\s+R\(G\) = ([0-9.eE+-]+)")),
            "R_plus_esp": float(num(r"R \+ ESP:\s+([0-9.eE+-]+)")),
            "paths": int(num(r"Paths enumerated:\s+(\d+)")),
            "nodes": int(num(r"Nodes processed:\s+(\d+)")),
            "waves": int(num(r"Kernel iterations:\s*(\d+)"))}


def test_cli_reproduces_the_published_block(golden, tmp_path):
    """The program prints the reference's result block; K9 and K10 match the published runs."""
    gdir = os.path.join(ROOT, "tests", "golden")
    for name, s, t in (("COMP9", 0, 8), ("COMP10-05", 0, 9)):
        path = os.path.join(gdir, golden["files"][name]["file"])
        out = subprocess.run([CLI, path, str(s), str(t), "--truncation_eps", "0", "--queue_capacity", "4194304"],
                             capture_output=True, text=True, timeout=300)
        assert out.returncode == 0, out.stderr
        b = parse_block(out.stdout)
        d = golden["published"][name]
        assert (b["paths"], b["nodes"], b["waves"]) == (d["paths"], d["nodes"], d["iterations"])
        assert abs(b["R"] - d["R"]) < 1e-11 and b["R_plus_esp"] == b["R"]
        assert "Graph loaded:" in out.stdout and "Launch config:" in out.stdout


def test_cli_flags(golden, oracle, load_golden_graph):
    gdir = os.path.join(ROOT, "tests", "golden")
    path = os.path.join(gdir, golden["files"]["COMP8"]["file"])
    out = subprocess.run([CLI, path, "0", "7", "--fork", "--queue_capacity", "1048576", "--truncation_eps", "0",
                          "--thresh_high", "1", "--thresh_low", "2", "--no_such_flag"],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    b = parse_block(out.stdout)
    o = oracle.run(load_golden_graph("COMP8"), 0, 7, branching="fork")
    assert (b["nodes"], b["paths"]) == (o.nodes, o.paths)
    out = subprocess.run([CLI, path, "0", "7", "--target_width", "1e-3", "--order", "maxmass"],
                         capture_output=True, text=True, timeout=300)
    b = parse_block(out.stdout)
    assert out.returncode == 0 and b["R_plus_esp"] - b["R"] <= 1e-3
    bad = subprocess.run([CLI, path, "0", "99"], capture_output=True, text=True, timeout=60)
    assert bad.returncode != 0 and "invalid" in bad.stderr
