"""GPU engine against the oracle and the reference's published results, through the C ABI.

Bars: counts (paths, nodes, leaves, dead ends, waves, widest wave) bit-exact;
R and ESP bit-exact against the oracle (FP64 path-order products, summed
exactly in 192-bit fixed point on both sides); R within 1e-12 relative of
brute force and of the reference's published values."""
import numpy as np
import pytest

from conftest import rel_close

pytestmark = pytest.mark.gpu

R_TOL = 1e-12


@pytest.fixture(scope="module")
def ctx(engine_lib):
    c = engine_lib.Context(0)
    yield c
    c.close()


def check_exact(r, o):
    assert r.paths == o.paths
    assert r.nodes == o.nodes
    assert r.leaves == o.leaves
    assert r.dead_ends == o.dead
    assert r.truncated == o.truncated
    assert r.iterations == o.waves
    assert r.max_queue_items == o.max_wave
    assert r.R == o.R, (r.R, o.R)
    assert r.esp == o.esp, (r.esp, o.esp)


@pytest.mark.parametrize("name", ["COMP8", "COMP8-03", "COMP9"])
def test_published_complete_graphs(ctx, golden, load_golden_graph, oracle, name):
    d = golden["published"][name]
    g = load_golden_graph(name)
    r = ctx.reliability(g, d["src"], d["dst"], capacity=1 << 22)
    assert (r.paths, r.nodes, r.iterations, r.max_queue_items) == (d["paths"], d["nodes"], d["iterations"],
                                                                    d["max_queue_items"])
    assert rel_close(r.R, d["R"], R_TOL)
    assert r.esp == 0.0
    check_exact(r, oracle.run(g, d["src"], d["dst"]))


def test_k10_published(ctx, golden, load_golden_graph):
    d = golden["published"]["COMP10-05"]
    g = load_golden_graph("COMP10-05")
    r = ctx.reliability(g, 0, 9, capacity=1 << 22)
    assert (r.paths, r.nodes, r.iterations, r.max_queue_items) == (d["paths"], d["nodes"], d["iterations"],
                                                                    d["max_queue_items"])
    assert rel_close(r.R, d["R"], R_TOL)


def test_k10_uniform_probabilities(ctx, oracle):
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(10, p_range=(0.5, 0.95), seed=2)
    r = ctx.reliability(g, 0, 9, capacity=1 << 22)
    check_exact(r, oracle.run(g, 0, 9, threads=4))


def test_golden_graphs_and_brute_force(ctx, golden, load_golden_graph, oracle):
    for name, f in golden["files"].items():
        if name.startswith("COMP"):
            continue
        g = load_golden_graph(name)
        s, t = f.get("src", 0), f.get("dst", g.n_nodes - 1)
        if name in golden["analytic"]:
            s, t = golden["analytic"][name]["src"], golden["analytic"][name]["dst"]
        if name == "test_kite":
            s, t = 0, 4
        r = ctx.reliability(g, s, t, capacity=1 << 20)
        check_exact(r, oracle.run(g, s, t))
        assert rel_close(r.R, oracle.brute(g, s, t), R_TOL), name


def test_grid_4x4_config(ctx, oracle):
    from relaibilitygpu_gb300 import graphs
    g = graphs.grid(4, 4, p=0.9)
    r = ctx.reliability(g, 0, 15, capacity=1 << 20)
    check_exact(r, oracle.run(g, 0, 15))
    assert rel_close(r.R, oracle.brute(g, 0, 15), R_TOL)


@pytest.mark.parametrize("seed", range(6))
def test_random_graphs_all_group_widths(ctx, oracle, seed):
    """n from 3 to 32 covers the 8-, 16- and 32-lane kernels; several mask widths."""
    from relaibilitygpu_gb300 import graphs
    rng = np.random.default_rng(seed)
    for n in (3, 7, 8, 9, 15, 16, 17, 24, 31, 32):
        m = int(min(n * (n - 1) // 2, n + rng.integers(0, 2 * n)))
        g = graphs.gnm(n, m, p_range=(0.4, 0.97), seed=int(rng.integers(1 << 30)))
        o = oracle.run(g, g.src, g.dst, max_nodes=3_000_000)
        if o.status != 0:
            continue
        r = ctx.reliability(g, g.src, g.dst, capacity=1 << 22)
        check_exact(r, o)


def test_eps_truncation_matches_oracle(ctx, load_golden_graph, oracle):
    g = load_golden_graph("COMP9")
    for eps in (1e-4, 1e-7):
        r = ctx.reliability(g, 0, 8, capacity=1 << 22, eps=eps)
        o = oracle.run(g, 0, 8, eps=eps)
        check_exact(r, o)
        assert r.esp == o.esp_truncated


def test_overflow_spills_and_brackets(ctx, golden, load_golden_graph):
    g = load_golden_graph("COMP9")
    exact = golden["published"]["COMP9"]["R"]
    r = ctx.reliability(g, 0, 8, capacity=20000)
    assert r.spilled > 0 and r.esp > 0
    assert r.R <= exact + 1e-15 <= r.R + r.esp + 2e-15
    assert r.paths == r.leaves + r.spilled


def test_capacity_one(ctx, load_golden_graph):
    g = load_golden_graph("COMP8")
    r = ctx.reliability(g, 0, 7, capacity=1)
    assert r.R <= 0.98257344961166381836 <= r.R + r.esp + 1e-15


def test_src_equals_dst_and_disconnected(ctx):
    from relaibilitygpu_gb300 import graphs
    r = ctx.reliability(graphs.complete(6, p=0.5), 3, 3)
    assert r.R == 1.0 and r.paths == 1 and r.nodes == 1
    g = graphs.from_edges(4, [(0, 1), (2, 3)], [0.9, 0.9])
    r = ctx.reliability(g, 0, 3)
    assert r.R == 0.0 and r.nodes == 1 and r.dead_ends == 1


def test_deterministic_edges(ctx, oracle):
    """p=1 edges start UP and p=0 edges start DOWN (main.cu:717-748)."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(7, p_range=(0.3, 0.9), seed=11)
    g.edge_p = g.edge_p.copy()
    g.edge_p[[0, 3, 9]] = 1.0
    g.edge_p[[1, 5]] = 0.0
    r = ctx.reliability(g, 0, 6)
    check_exact(r, oracle.run(g, 0, 6))
    assert rel_close(r.R, oracle.brute(g, 0, 6), R_TOL)


def test_one_shot_entry_point(engine_lib, load_golden_graph):
    g = load_golden_graph("test_bridge")
    r = engine_lib.reliability(g, 0, 3)
    assert rel_close(r.R, 0.835, 1e-14)


def test_directed_graphs_all_engines(ctx, oracle):
    """'D' graphs (every arc its own edge, searches follow arcs) on the whole-GPU wave engine,
    the warp engine and the wide engines, against the oracle."""
    from relaibilitygpu_gb300 import graphs
    rng = np.random.default_rng(9)
    compared = 0
    for n in (8, 14, 20, 24, 48):
        arcs = sorted({(int(a), int(b)) for a, b in rng.integers(0, n, size=(4 * n, 2)) if a != b})
        g = graphs.from_arcs(n, arcs, rng.uniform(0.6, 0.97, size=len(arcs)))
        s, t = 0, n - 1
        o = oracle.run(g, s, t, max_nodes=3_000_000, threads=4)
        if o.status == 0:
            r = ctx.reliability(g, s, t, capacity=1 << 22)
            check_exact(r, o)
        for shift in (-1, 1):
            nb = 64 if shift >= 0 else 1
            o2 = oracle.run(g, s, t, target_width=1e-4, bucket_shift=shift, n_buckets=nb, threads=4)
            r2 = ctx.reliability(g, s, t, capacity=1 << 22, target_width=1e-4, bucket_shift=shift, n_buckets=64,
                                 order="maxmass")
            if r2.spilled:
                continue          # larger than one warp's queue: a valid bracket, not the oracle's run
            assert (r2.nodes, r2.leaves, r2.dead_ends, r2.iterations) == (o2.nodes, o2.leaves, o2.dead, o2.waves)
            assert r2.R == o2.R and r2.esp == o2.esp
            compared += 1
    assert compared >= 6
