"""Pin the CPU oracle against the reference: published run logs, analytic
values, brute force, and the reference's own seq.cpp / cpu_reference.cpp
outputs (tests/golden/golden.json, made by tests/golden/make_golden.py)."""
import pytest

from conftest import rel_close

SMALL_PUBLISHED = ["COMP8", "COMP8-03", "COMP9"]


@pytest.mark.parametrize("name", SMALL_PUBLISHED)
def test_published_counts_main_cu(golden, load_golden_graph, oracle, name):
    """main.cu semantics: nodes include dead ends; waves and widest wave match the logs."""
    d = golden["published"][name]
    g = load_golden_graph(name)
    r = oracle.run(g, d["src"], d["dst"], rule="level", order="waves")
    assert r.paths == d["paths"]
    assert r.nodes == d["nodes"]
    assert r.waves == d["iterations"]
    assert r.max_wave == d["max_queue_items"]
    # COMP8-03's published FP64 value is a log-space sum (seq.cpp); the linear
    # product agrees to ~4e-14 relative and brute force to ~1e-15
    assert rel_close(r.R, d["R"], 1e-12)
    assert r.esp == 0.0


def test_published_k10_counts(golden, load_golden_graph, oracle):
    d = golden["published"]["COMP10-05"]
    g = load_golden_graph("COMP10-05")
    r = oracle.run(g, 0, 9, rule="level", order="waves", threads=4)
    assert (r.paths, r.nodes, r.waves, r.max_wave) == (d["paths"], d["nodes"], d["iterations"], d["max_queue_items"])
    assert rel_close(r.R, d["R"], 1e-15)


@pytest.mark.parametrize("name", SMALL_PUBLISHED)
def test_seq_cpp_semantics(golden, load_golden_graph, oracle, name):
    """seq.cpp semantics (FIFO parent, pre-push check): iterations = paths = published."""
    d = golden["published"][name]
    g = load_golden_graph(name)
    r = oracle.run(g, d["src"], d["dst"], rule="fifo", precheck=True, order="heap")
    assert r.nodes == d["paths"]
    assert r.paths == d["paths"]


def test_seq_ref_random_graphs(golden, load_golden_graph, oracle):
    """The reference's seq.cpp built from source on seeded random graphs."""
    seq = golden["seq_ref"]
    assert len(seq) >= 20
    for name, d in seq.items():
        g = load_golden_graph(name)
        r = oracle.run(g, d["src"], d["dst"], rule="fifo", precheck=True, order="heap")
        assert r.nodes == d["iterations"], name
        assert r.paths == d["paths"], name
        assert rel_close(r.R, d["R"], 1e-12), (name, r.R, d["R"])


def test_cpu_reference_tiny(golden, load_golden_graph, oracle):
    """workingPad/cpu_reference.cpp reads p as float: agreement to float precision."""
    for name, d in golden["cpu_reference"].items():
        g = load_golden_graph(name)
        r = oracle.run(g, d["src"], d["dst"])
        assert abs(r.R - d["R"]) < 1e-6, name


def test_analytic(golden, load_golden_graph, oracle):
    for name, d in golden["analytic"].items():
        g = load_golden_graph(name)
        for rule in ("level", "fifo"):
            r = oracle.run(g, d["src"], d["dst"], rule=rule)
            assert rel_close(r.R, d["R"], 1e-14), (name, rule, r.R)


def test_brute_force_agrees(golden, load_golden_graph, oracle):
    names = [n for n in golden["files"] if n.startswith(("gnm", "grid", "kn", "test_", "cycle", "temp"))]
    for name in names:
        g = load_golden_graph(name)
        f = golden["files"][name]
        s, t = f.get("src", 0), f.get("dst", g.n_nodes - 1)
        if name in golden["analytic"]:
            s, t = golden["analytic"][name]["src"], golden["analytic"][name]["dst"]
        if name == "test_kite":
            s, t = 0, 4
        b = oracle.brute(g, s, t)
        for rule in ("level", "fifo"):
            r = oracle.run(g, s, t, rule=rule)
            assert rel_close(r.R, b, 1e-13), (name, rule, r.R, b)


def test_grid4x4_config(oracle):
    from relaibilitygpu_gb300 import graphs
    g = graphs.grid(4, 4, p=0.9)
    b = oracle.brute(g, 0, 15)
    r = oracle.run(g, 0, 15)
    assert rel_close(r.R, b, 1e-14)
    assert rel_close(b, 0.97504634957706637, 1e-14)


def test_orders_agree_when_exhaustive(load_golden_graph, oracle):
    g = load_golden_graph("COMP8")
    base = oracle.run(g, 0, 7, order="waves")
    for kw in (dict(order="heap"), dict(order="dfs"), dict(order="waves", bucket_shift=2, n_buckets=64),
               dict(order="waves", threads=3)):
        r = oracle.run(g, 0, 7, **kw)
        assert (r.paths, r.nodes, r.leaves, r.dead) == (base.paths, base.nodes, base.leaves, base.dead), kw
        assert rel_close(r.R, base.R, 1e-14)


def test_truncation_brackets(golden, load_golden_graph, oracle):
    """Truncated runs bracket the exhaustive value: R <= R_exact <= R + ESP."""
    g = load_golden_graph("COMP9")
    exact = oracle.run(g, 0, 8).R
    for kw in (dict(eps=1e-6), dict(capacity=5000), dict(bucket_shift=2, n_buckets=128, target_width=1e-4),
               dict(order="heap", capacity=300), dict(bucket_shift=1, n_buckets=64, target_width=1e-2)):
        r = oracle.run(g, 0, 8, **kw)
        assert r.R <= exact + 1e-15, kw
        assert exact <= r.R + r.esp + 1e-15, kw
        if kw.get("target_width"):
            assert r.status == 1 and r.esp <= kw["target_width"]


def test_k15_published_bracket(golden, load_golden_graph, oracle):
    """A truncated K15 p=0.5 run overlaps the reference's truncated bracket."""
    d = golden["published"]["COMP15-05_bracket"]
    g = load_golden_graph("COMP15-05")
    r = oracle.run(g, 0, 14, bucket_shift=2, n_buckets=256, target_width=2e-3, threads=4)
    assert r.status == 1
    assert r.R <= d["hi"] and d["lo"] <= r.R + r.esp


def test_bucket_function(oracle):
    assert oracle.bucket(1.0, 2, 256) == 0
    assert oracle.bucket(0.5, 2, 256) == 4
    assert oracle.bucket(0.75, 2, 256) == 2
    assert oracle.bucket(1e-300, 2, 256) == 255
    assert oracle.bucket(0.3, -1, 1) == 0
    ms = [1.0, 0.9, 0.7, 0.5, 0.26, 0.01, 1e-5]
    bs = [oracle.bucket(m, 3, 512) for m in ms]
    assert bs == sorted(bs)


def test_src_equals_dst(oracle):
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(5, p=0.5)
    r = oracle.run(g, 2, 2)
    assert r.R == 1.0 and r.paths == 1 and r.nodes == 1


def test_disconnected(oracle):
    from relaibilitygpu_gb300 import graphs
    g = graphs.from_edges(4, [(0, 1), (2, 3)], [0.9, 0.9])
    r = oracle.run(g, 0, 3)
    assert r.R == 0.0 and r.nodes == 1 and r.dead == 1 and r.paths == 0


def test_batch_runner_matches_single(oracle):
    """og_run_batch (reused per-thread storage) gives the single-instance results."""
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(15, p_range=(0.9, 0.99), seed=s) for s in range(40)]
    gs += [graphs.grid(3, 4, p_range=(0.5, 0.95), seed=s) for s in range(10)]
    srcs = [0] * len(gs)
    dsts = [g.n_nodes - 1 for g in gs]
    kw = dict(bucket_shift=2, n_buckets=256, target_width=1e-6)
    res = oracle.run_batch(oracle.BatchArgs(gs, srcs, dsts), threads=3, **kw)
    for i, g in enumerate(gs):
        o = oracle.run(g, srcs[i], dsts[i], **kw)
        r = res[i]
        assert (r.nodes, r.leaves, r.dead, r.waves, r.max_wave, r.queued) == (o.nodes, o.leaves, o.dead, o.waves,
                                                                             o.max_wave, o.queued)
        assert r.R == o.R and r.esp == o.esp


def test_fork_branching_is_exact(load_golden_graph, oracle):
    """Fork branching (main.cu:303-430 with FORK_BEST_EDGE) is a different decomposition with the
    same R: exhaustive runs agree with brute force; truncated runs bracket it."""
    from relaibilitygpu_gb300 import graphs
    cases = [(load_golden_graph("COMP8"), 0, 7), (load_golden_graph("test_kite"), 0, 4),
             (graphs.grid(3, 4, p_range=(0.5, 0.95), seed=3), 0, 11),
             (graphs.gnm(9, 16, p_range=(0.3, 0.95), seed=5), None, None)]
    for g, s, t in cases:
        s = g.src if s is None else s
        t = g.dst if t is None else t
        exact = oracle.brute(g, s, t)
        for order, kw in (("waves", {}), ("waves", dict(bucket_shift=2, n_buckets=64)), ("heap", {})):
            r = oracle.run(g, s, t, order=order, branching="fork", **kw)
            assert r.status == 0 and r.esp == 0.0
            assert abs(r.R - exact) <= 1e-13 * max(exact, 1e-300)
            # every pop is a leaf, a dead end or a fork with two children, and every child is popped
            assert r.paths == r.leaves and r.pushes % 2 == 0
            assert r.nodes == r.leaves + r.dead + r.pushes // 2 == 1 + r.pushes
        r = oracle.run(g, s, t, branching="fork", bucket_shift=1, n_buckets=64, target_width=1e-3)
        assert r.R <= exact + 1e-15 <= r.R + r.esp + 1e-15 and r.esp <= 1e-3


def test_fork_branching_counts_by_hand():
    """A 3-edge path s-a-t plus the edge s-t: the fork picks the most reliable UNKNOWN edge of the
    optimistic path s-t first (the direct edge), then the path s-a-t with its best edge."""
    import oracle
    from relaibilitygpu_gb300 import graphs
    g = graphs.from_edges(3, [(0, 1), (1, 2), (0, 2)], [0.9, 0.8, 0.7])
    r = oracle.run(g, 0, 2, branching="fork")
    # pops: root (s-t unknown -> fork on (0,2)); up child: connected leaf; down child: path 0-1-2,
    # fork on (0,1) p=0.9: its down child is dead, its up child forks on (1,2): up leaf, down dead
    assert (r.nodes, r.leaves, r.dead, r.pushes) == (7, 2, 2, 6)
    assert abs(r.R - (0.7 + 0.3 * 0.9 * 0.8)) < 1e-15


def test_directed_graphs(oracle, tmp_path):
    """'D' files give every arc its own edge id (seq/GraphRP.h:131-145); searches follow arcs."""
    import numpy as np
    from relaibilitygpu_gb300 import graphs
    # 0->1->2 with a back arc 2->1 and an arc 2->0 that cannot help a 0->2 path
    g = graphs.from_arcs(3, [(0, 1), (1, 2), (2, 1), (2, 0)], [0.9, 0.8, 0.5, 0.7])
    assert (g.n_edges, g.n_arcs) == (4, 4)
    r = oracle.run(g, 0, 2)
    assert abs(r.R - 0.9 * 0.8) < 1e-15 and abs(oracle.brute(g, 0, 2) - 0.72) < 1e-15
    # the reverse direction needs 2->0 or 2->1->? : only 2->0
    assert abs(oracle.run(g, 2, 0).R - 0.7) < 1e-15
    text = graphs.format_graph(g, "D")
    g2 = graphs.parse_graph_text(text)
    assert np.array_equal(g2.edge_id, g.edge_id) and np.array_equal(g2.edge_p, g.edge_p)
    assert abs(oracle.run(g2, 0, 2).R - 0.72) < 1e-15
    # a random directed graph: the decomposition equals brute force, with both parent rules
    rng = np.random.default_rng(3)
    arcs = sorted({(int(a), int(b)) for a, b in rng.integers(0, 8, size=(30, 2)) if a != b})
    dg = graphs.from_arcs(8, arcs, rng.uniform(0.4, 0.95, size=len(arcs)))
    exact = oracle.brute(dg, 0, 7)
    for rule in ("level", "fifo"):
        assert abs(oracle.run(dg, 0, 7, rule=rule).R - exact) <= 1e-13


def test_k_terminal_decomposition(load_golden_graph, oracle):
    """K-terminal reliability (every terminal joined to terminals[0]) by the same disjoint
    decomposition over the BFS tree: exact against brute force; two terminals give the
    two-terminal run exactly; truncated runs bracket it."""
    from relaibilitygpu_gb300 import graphs
    g = load_golden_graph("COMP8")
    two = oracle.run(g, 0, 7)
    k2 = oracle.run(g, 0, 0, terminals=[0, 7])
    assert (k2.R, k2.nodes, k2.paths, k2.waves) == (two.R, two.nodes, two.paths, two.waves)
    cases = [(graphs.complete(7, p_range=(0.5, 0.95), seed=2), [0, 3, 6]),
             (graphs.grid(3, 4, p_range=(0.6, 0.97), seed=4), [0, 5, 11, 3]),
             (graphs.gnm(9, 15, p_range=(0.4, 0.95), seed=6), [2, 0, 8, 4, 7]),
             (graphs.from_arcs(4, [(0, 1), (1, 2), (2, 3), (3, 0), (0, 2)], [0.9, 0.8, 0.7, 0.6, 0.5]), [0, 2, 3])]
    for gg, term in cases:
        exact = oracle.brute_k(gg, term)
        for kw in ({}, dict(bucket_shift=1, n_buckets=64), dict(order="heap")):
            r = oracle.run(gg, 0, 0, terminals=term, **kw)
            assert r.status == 0 and abs(r.R - exact) <= 1e-13, (term, kw, r.R, exact)
        t = oracle.run(gg, 0, 0, terminals=term, target_width=1e-3, bucket_shift=1, n_buckets=64)
        assert t.R <= exact + 1e-15 <= t.R + t.esp + 1e-15
    assert abs(oracle.brute_k(graphs.complete(5, p=0.5), [1]) - 1.0) < 1e-15   # one terminal


def test_batch_runner_mixed_mask_widths(oracle):
    """og_run_batch keeps one set of queue vectors per thread for all its instances: records of a
    wider mask after a narrower one must fit the storage (it counts words, not records), and every
    instance equals its own og_run."""
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.grid(4, 4, p_range=(0.6, 0.95), seed=1), graphs.complete(12, p_range=(0.5, 0.95), seed=2),
          graphs.grid(3, 3, p=0.9), graphs.complete(14, p_range=(0.7, 0.99), seed=3)] * 2
    srcs = [0] * len(gs)
    dsts = [g.n_nodes - 1 for g in gs]
    kw = dict(bucket_shift=-1, n_buckets=1, target_width=1e-7, max_nodes=400_000)
    res = oracle.run_batch(oracle.BatchArgs(gs, srcs, dsts), threads=1, **kw)
    assert max(res[i].max_wave for i in range(len(gs))) > 4096
    for i, g in enumerate(gs):
        o = oracle.run(g, srcs[i], dsts[i], **kw)
        r = res[i]
        assert (r.nodes, r.waves, r.max_wave, r.queued, r.R, r.esp) == (o.nodes, o.waves, o.max_wave, o.queued,
                                                                         o.R, o.esp)
