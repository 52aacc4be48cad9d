"""One-lane-per-subproblem warp kernel (nr_lane.cuh) against the oracle and the
lane-group kernel (nr_warp.cuh).

Truncated runs follow the oracle's wave schedule, so every count (waves, widest
wave, nodes, leaves, dead ends, truncated, queued) is bit-exact and R and ESP
(exact fixed-point sums) are equal.  Exhaustive batches run page by page; their
totals do not depend on the order, so they equal the oracle's too."""
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("R", "esp", "nodes", "leaves", "dead_ends", "truncated", "spilled", "paths", "iterations",
          "max_queue_items", "queued", "stop")
TWO_SLOT = ("lane2", "block")      # breadth-first waves: the two-slot kernel, or its hand-over


@pytest.fixture(scope="module")
def ctx(engine_lib):
    c = engine_lib.Context(0)
    yield c
    c.close()


def mixed_batch():
    """Instances the lane kernel takes (undirected simple, n <= 16) and some it leaves to the
    lane groups (n > 16, directed, parallel edges)."""
    from relaibilitygpu_gb300 import graphs
    gs, st = [], []
    for s in range(48):
        gs.append(graphs.complete(15, p_range=(0.9, 0.99), seed=s)); st.append((0, 14))
    for s in range(8):
        gs.append(graphs.complete(8, p_range=(0.5, 0.95), seed=100 + s)); st.append((0, 7))
        gs.append(graphs.grid(3, 4, p_range=(0.6, 0.97), seed=200 + s)); st.append((0, 11))
        gs.append(graphs.grid(4, 4, p_range=(0.7, 0.99), seed=300 + s)); st.append((0, 15))
        g = graphs.gnm(12, 30, p_range=(0.8, 0.99), seed=400 + s); gs.append(g); st.append((g.src, g.dst))
        gs.append(graphs.complete(20, p_range=(0.9, 0.99), seed=500 + s)); st.append((0, 19))
    # edge cases: src == dst, an isolated dst, certain edges (p = 0 and p = 1), two nodes
    gs.append(graphs.complete(6, p=0.7)); st.append((3, 3))
    gs.append(graphs.from_edges(5, [(0, 1), (1, 2), (2, 0), (3, 1)], [0.9, 0.8, 0.7, 0.6])); st.append((0, 4))
    gs.append(graphs.from_edges(6, [(0, 1), (1, 5), (0, 2), (2, 5), (1, 2), (0, 5)], [1.0, 0.9, 0.0, 0.8, 1.0, 0.5]))
    st.append((0, 5))
    gs.append(graphs.from_edges(2, [(0, 1)], [0.75])); st.append((0, 1))
    # parallel edges and a directed graph: lane groups
    gs.append(graphs.from_edges(4, [(0, 1), (0, 1), (1, 3), (0, 2), (2, 3)], [0.9, 0.8, 0.7, 0.6, 0.95]))
    st.append((0, 3))
    gs.append(graphs.from_arcs(6, [(0, 1), (1, 2), (2, 5), (0, 3), (3, 4), (4, 5), (1, 4), (4, 1)],
                               [0.9, 0.8, 0.7, 0.85, 0.75, 0.95, 0.6, 0.65]))
    st.append((0, 5))
    return gs, [s for s, _ in st], [t for _, t in st]


def lane_expected(g, max_n=16):
    """n <= max_n and an undirected simple graph: every edge id on exactly the two arcs u -> v and
    v -> u, no self-loop, no ordered pair twice.  (The one-slot lane kernel takes up to 16 nodes,
    the two-slot kernel of breadth-first waves up to 32.)"""
    import numpy as np
    if g.n_nodes > max_n:
        return False
    tails = np.repeat(np.arange(g.n_nodes), np.diff(g.row_ptr))
    arcs = list(zip(tails.tolist(), g.col_idx.tolist(), g.edge_id.tolist()))
    if len({(u, v) for u, v, _ in arcs}) != len(arcs) or any(u == v for u, v, _ in arcs):
        return False
    by_id = {}
    for u, v, e in arcs:
        by_id.setdefault(e, []).append((u, v))
    return len(by_id) == g.n_edges and all(len(a) == 2 and a[0] == a[1][::-1] for a in by_id.values())


@pytest.mark.parametrize("target,shift", [(1e-6, -1), (1e-6, 0), (1e-9, 2), (1e-3, 1)])
def test_lane_kernel_wave_schedule(ctx, oracle, target, shift):
    """The largest queue of these runs is 27K records (oracle): 64K per warp never spills, and a
    run that spilled more mass than its target could not meet it and would run on to the empty
    queue."""
    gs, srcs, dsts = mixed_batch()
    nb = 64 << max(shift, 0)
    lane = ctx.reliability_batch(gs, srcs, dsts, target_width=target, bucket_shift=shift, n_buckets=nb,
                                 capacity=1 << 16)
    group = ctx.reliability_batch(gs, srcs, dsts, target_width=target, bucket_shift=shift, n_buckets=nb,
                                  capacity=1 << 16, small_kernel="group")
    # one bucket: two instances per warp by default; the one-instance lane kernel beside it
    one = ctx.reliability_batch(gs, srcs, dsts, target_width=target, bucket_shift=shift, n_buckets=nb,
                                capacity=1 << 16, small_kernel="lane1")
    # one bucket: the two-slot kernel, or the block kernel it hands an instance to once a wave
    # outgrows the warp
    lane_names = TWO_SLOT if shift < 0 else ("lane",)
    if shift < 0:                                 # four instances a warp instead of the default two
        two = ctx.reliability_batch(gs, srcs, dsts, target_width=target, bucket_shift=shift, n_buckets=nb,
                                    capacity=1 << 16, lane_slots=4)
        for i, (g, a, d) in enumerate(zip(gs, lane, two)):
            assert d.kernel in (TWO_SLOT if lane_expected(g) else ("group",)), i   # 17..32 nodes: two slots only
            for f in FIELDS:
                assert getattr(a, f) == getattr(d, f), (i, f)
    for i, (g, a, b, c) in enumerate(zip(gs, lane, group, one)):
        assert a.engine == "warp" and b.engine == "warp" and a.spilled == 0
        assert a.kernel in (lane_names if lane_expected(g, 32 if shift < 0 else 16) else ("group",)), i
        assert b.kernel == "group" and c.kernel == ("lane" if lane_expected(g) else "group")
        for f in FIELDS:
            assert getattr(a, f) == getattr(b, f), (i, f, getattr(a, f), getattr(b, f))
            assert getattr(c, f) == getattr(b, f), (i, f, getattr(c, f), getattr(b, f))
        if i % 5 == 0 or i >= len(gs) - 6:
            o = oracle.run(g, srcs[i], dsts[i], target_width=target, bucket_shift=shift,
                           n_buckets=nb if shift >= 0 else 1)
            assert (a.nodes, a.leaves, a.dead_ends, a.iterations, a.max_queue_items, a.queued) == \
                (o.nodes, o.leaves, o.dead, o.waves, o.max_wave, o.queued), i
            assert a.R == o.R and a.esp == o.esp, i


def test_lane_kernel_exhaustive_pages_and_truncation(ctx, oracle):
    """Exhaustive batches (page mode) and eps truncation: the oracle's totals and exact sums."""
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(8, p_range=(0.5, 0.95), seed=s) for s in range(6)] + \
         [graphs.grid(3, 4, p_range=(0.6, 0.97), seed=s) for s in range(6)] + \
         [graphs.complete(9, p=0.5), graphs.complete(9, p_range=(0.5, 0.95), seed=2)]
    srcs = [0] * len(gs)
    dsts = [g.n_nodes - 1 for g in gs]
    for eps in (0.0, 1e-6):
        res = ctx.reliability_batch(gs, srcs, dsts, eps=eps, capacity=1 << 16)
        for g, s, t, r in zip(gs, srcs, dsts, res):
            o = oracle.run(g, s, t, eps=eps)
            assert r.kernel == "lane" and r.engine == "warp"
            assert (r.nodes, r.leaves, r.dead_ends, r.truncated, r.paths) == \
                (o.nodes, o.leaves, o.dead, o.truncated, o.paths)
            assert r.R == o.R and r.esp == o.esp


def test_lane_kernel_spills_budget_and_handover(ctx, oracle):
    """A full queue spills into ESP (a bracket); a pop budget stops between waves like the
    lane groups; an exhaustive instance larger than its warp's queue goes to the whole-GPU
    engine and is still exact."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(9, p_range=(0.6, 0.97), seed=5)
    exact = oracle.run(g, 0, 8)
    r = ctx.reliability(g, 0, 8, target_width=1e-14, bucket_shift=1, n_buckets=128, capacity=128)
    assert r.kernel == "lane" and r.spilled > 0
    assert r.R <= exact.R + 1e-15 and exact.R <= r.R + r.esp + 1e-12
    k12 = graphs.complete(12, p_range=(0.7, 0.99), seed=5)
    opts = dict(target_width=1e-12, bucket_shift=1, n_buckets=128, max_nodes=3000)
    a = ctx.reliability(k12, 0, 11, **opts)
    b = ctx.reliability(k12, 0, 11, small_kernel="group", **opts)
    assert a.stop == 3 and a.kernel == "lane" and b.kernel == "group"
    for f in FIELDS:
        assert getattr(a, f) == getattr(b, f), f
    big = graphs.complete(10, p=0.5)           # 14.9M subproblems: past the warp engine's 2^21 budget
    res = ctx.reliability_batch([big, g], [0, 0], [9, 8], capacity=1 << 12)
    o = oracle.run(big, 0, 9, threads=8)
    assert res[0].engine == "grid" and (res[0].nodes, res[0].paths, res[0].R) == (o.nodes, o.paths, o.R)
    assert res[1].kernel == "lane" and res[1].R == exact.R and res[1].nodes == exact.nodes


def test_two_slot_kernel_budget_spills_and_uneven_batches(ctx, oracle):
    """Breadth-first waves (two instances a warp): a node budget stops each instance between its
    waves exactly as the lane-group kernel does; a slot whose half of the pages is full spills into
    ESP and the bracket holds; batches of 1, 2, 3 and 33 instances (empty slots, a warp with one
    instance) give the oracle's results."""
    from relaibilitygpu_gb300 import graphs
    k12 = graphs.complete(12, p_range=(0.7, 0.99), seed=5)
    opts = dict(target_width=1e-12, bucket_shift=-1, n_buckets=64, max_nodes=3000)
    a = ctx.reliability(k12, 0, 11, **opts)
    b = ctx.reliability(k12, 0, 11, small_kernel="group", **opts)
    assert a.stop == 3 and a.kernel in TWO_SLOT and b.kernel == "group"
    for f in FIELDS:
        assert getattr(a, f) == getattr(b, f), f
    g = graphs.complete(9, p_range=(0.6, 0.97), seed=5)
    exact = oracle.run(g, 0, 8)
    r = ctx.reliability(g, 0, 8, target_width=1e-14, bucket_shift=-1, n_buckets=64, capacity=256)
    assert r.kernel == "lane2" and r.spilled > 0
    assert r.R <= exact.R + 1e-15 and exact.R <= r.R + r.esp + 1e-12
    for m in (1, 2, 3, 33):
        gs = [graphs.complete(8 + s % 6, p_range=(0.8, 0.99), seed=700 + s) for s in range(m)]
        res = ctx.reliability_batch(gs, [0] * m, [x.n_nodes - 1 for x in gs], target_width=1e-7,
                                    bucket_shift=-1, n_buckets=64, capacity=1 << 14)
        for x, rr in zip(gs, res):
            o = oracle.run(x, 0, x.n_nodes - 1, target_width=1e-7)
            assert rr.kernel in TWO_SLOT and rr.spilled == 0
            assert (rr.nodes, rr.iterations, rr.max_queue_items, rr.queued) == (o.nodes, o.waves, o.max_wave, o.queued)
            assert rr.R == o.R and rr.esp == o.esp


def lane32_batch():
    """Undirected simple graphs of 17..32 nodes (32-bit rows in the two-slot kernel), mask widths
    1..8 blocks, and edge cases: certain edges (p = 0 and 1: the root's rows are gathered), src ==
    dst, an unreachable dst, a two-node path inside a large node set."""
    from relaibilitygpu_gb300 import graphs
    gs, st = [], []
    for s in range(6):
        for r, c in ((4, 5), (5, 5), (5, 6), (6, 5), (4, 8)):
            g = graphs.grid(r, c, p_range=(0.8, 0.99), seed=900 + 10 * s + r * c)
            gs.append(g); st.append((0, g.n_nodes - 1))
        g = graphs.gnm(20, 60, p_range=(0.8, 0.99), seed=950 + s); gs.append(g); st.append((g.src, g.dst))
        g = graphs.gnm(28, 84, p_range=(0.85, 0.99), seed=960 + s); gs.append(g); st.append((g.src, g.dst))
        gs.append(graphs.complete(20, p_range=(0.9, 0.99), seed=970 + s)); st.append((0, 19))
    gs.append(graphs.complete(25, p_range=(0.9, 0.99), seed=980)); st.append((0, 24))
    gs.append(graphs.complete(32, p_range=(0.95, 0.99), seed=981)); st.append((3, 30))
    g = graphs.grid(5, 5, p_range=(0.8, 0.99), seed=982)
    p = g.edge_p.copy(); p[3] = 0.0; p[7] = 1.0; p[11] = 0.0
    gs.append(graphs.from_edges(25, g.edge_list(), p)); st.append((0, 24))
    gs.append(graphs.grid(4, 5, p_range=(0.8, 0.99), seed=983)); st.append((7, 7))
    gs.append(graphs.from_edges(20, [(i, i + 1) for i in range(18)] + [(0, 5)], [0.9] * 19)); st.append((0, 19))
    gs.append(graphs.from_edges(30, [(0, 29)] + [(i, i + 1) for i in range(1, 28)], [0.8] * 28)); st.append((0, 29))
    return gs, [a for a, _ in st], [b for _, b in st]


@pytest.mark.parametrize("target,budget,border", [(1e-6, 0, "src"), (1e-9, 4000, "src"), (1e-7, 0, "p_asc"),
                                                  (1e-5, 0, "dst")])
def test_two_slot_kernel_32_bit_rows(ctx, oracle, target, budget, border):
    """Graphs of 17..32 nodes in breadth-first waves run in the two-slot lane kernel with 32-bit
    rows; every field equals the lane-group kernel's and the oracle's (waves, widest wave, counts,
    queue, exact sums), with budgets and branch orders.  Runs whose queue filled (each slot has
    the lane-group kernel's pages, but the kernels choose different children to spill) are
    brackets of the same value."""
    gs, srcs, dsts = lane32_batch()
    opts = dict(target_width=target, bucket_shift=-1, n_buckets=64, capacity=1 << 18, max_nodes=budget,
                branch_order=border)
    lane = ctx.reliability_batch(gs, srcs, dsts, **opts)
    group = ctx.reliability_batch(gs, srcs, dsts, small_kernel="group", **opts)
    compared = 0
    for i, (g, a, b) in enumerate(zip(gs, lane, group)):
        assert a.kernel in (TWO_SLOT if lane_expected(g, 32) else ("group",)) and b.kernel == "group", i
        if a.spilled or b.spilled:            # a full queue (the large grids at 1e-6): brackets of
            assert max(a.R, b.R) <= min(a.R + a.esp, b.R + b.esp) + 1e-15, i   # the same value
            continue
        for f in FIELDS:
            assert getattr(a, f) == getattr(b, f), (i, f, getattr(a, f), getattr(b, f))
        if i % 3 == 0 or i >= len(gs) - 6:
            o = oracle.run(g, srcs[i], dsts[i], target_width=target, max_nodes=budget, branch_order=border)
            assert (a.nodes, a.leaves, a.dead_ends, a.iterations, a.max_queue_items, a.queued) == \
                (o.nodes, o.leaves, o.dead, o.waves, o.max_wave, o.queued), i
            assert a.R == o.R and a.esp == o.esp, i
            compared += 1
    assert compared >= 12


def test_two_slot_kernel_32_bit_rows_spills(ctx, oracle):
    """A 32-bit-row instance whose half of the warp's pages fills spills into ESP; the bracket
    holds (exact R of a 4 x 5 grid by the oracle)."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.grid(4, 5, p_range=(0.6, 0.95), seed=3)
    exact = oracle.run(g, 0, 19, threads=8)
    r = ctx.reliability(g, 0, 19, target_width=1e-15, bucket_shift=-1, n_buckets=64, capacity=256)
    assert r.kernel == "lane2" and r.spilled > 0
    assert r.R <= exact.R + 1e-15 and exact.R <= r.R + r.esp + 1e-12


def test_whole_gpu_lane_kernel(ctx, oracle):
    """Single exhaustive (and eps-truncated) runs of undirected simple graphs of <= 16 nodes take
    the whole-GPU wave engine with one lane per subproblem; counts, waves, widest wave and exact
    sums equal the lane-group version's (small_kernel="group") and the oracle's, with branch
    orders; a capacity overflow spills into a bracket."""
    from relaibilitygpu_gb300 import graphs
    cases = [(graphs.complete(8, p=0.5), 0, 7), (graphs.complete(9, p_range=(0.5, 0.95), seed=3), 0, 8),
             (graphs.grid(3, 4, p_range=(0.6, 0.97), seed=4), 0, 11), (graphs.grid(4, 4, p=0.9), 0, 15),
             (graphs.gnm(14, 30, p_range=(0.7, 0.99), seed=5), 2, 11),
             (graphs.from_edges(6, [(0, 1), (1, 5), (0, 2), (2, 5), (1, 2), (0, 5)], [1.0, 0.9, 0.0, 0.8, 1.0, 0.5]), 0, 5),
             (graphs.complete(6, p=0.7), 3, 3),
             (graphs.from_edges(5, [(0, 1), (1, 2), (2, 0), (3, 1)], [0.9, 0.8, 0.7, 0.6]), 0, 4)]
    for g, s, t in cases:
        for eps, border in ((0.0, "src"), (1e-6, "src"), (0.0, "p_asc"), (1e-7, "dst")):
            a = ctx.reliability(g, s, t, capacity=1 << 22, eps=eps, branch_order=border)
            b = ctx.reliability(g, s, t, capacity=1 << 22, eps=eps, branch_order=border, small_kernel="group")
            assert a.engine == "grid" and b.engine == "grid" and a.kernel == "lane" and b.kernel == ""
            for f in ("R", "esp", "nodes", "leaves", "dead_ends", "truncated", "spilled", "paths", "iterations",
                      "max_queue_items"):
                assert getattr(a, f) == getattr(b, f), (g.n_nodes, eps, border, f)
            o = oracle.run(g, s, t, eps=eps, branch_order=border)
            assert (a.nodes, a.leaves, a.dead_ends, a.truncated, a.iterations, a.max_queue_items) == \
                (o.nodes, o.leaves, o.dead, o.truncated, o.waves, o.max_wave)
            assert a.R == o.R and a.esp == o.esp
    # the reference's published K10 p=0.5 run: 14,866,064 subproblems in 38 waves, widest 1,596,000
    k10 = graphs.complete(10, p=0.5)
    r = ctx.reliability(k10, 0, 9, capacity=1 << 22)
    assert r.kernel == "lane" and (r.nodes, r.iterations, r.max_queue_items) == (14866064, 38, 1596000)
    g = graphs.complete(9, p_range=(0.6, 0.97), seed=5)
    exact = oracle.run(g, 0, 8)
    r = ctx.reliability(g, 0, 8, capacity=2000)
    assert r.kernel == "lane" and r.spilled > 0
    assert r.R <= exact.R + 1e-15 and exact.R <= r.R + r.esp + 1e-12


def test_whole_gpu_lane_kernel_32_bit_rows(ctx, oracle):
    """17..32-node undirected simple graphs in the whole-GPU wave engine take one lane per
    subproblem with 32-bit rows: exhaustive and eps-truncated runs, branch orders, certain edges;
    every count, wave and exact sum equals the lane-group version's and the oracle's."""
    from relaibilitygpu_gb300 import graphs
    g5 = graphs.grid(4, 5, p_range=(0.8, 0.99), seed=21)
    p = g5.edge_p.copy(); p[2] = 0.0; p[9] = 1.0
    cases = [(graphs.grid(4, 5, p=0.9), 0, 19), (graphs.grid(3, 6, p_range=(0.7, 0.99), seed=22), 0, 17),
             (graphs.gnm(20, 34, p_range=(0.8, 0.99), seed=1), None, None),
             (graphs.from_edges(20, g5.edge_list(), p), 0, 19),
             (graphs.complete(20, p_range=(0.3, 0.7), seed=23), 0, 19)]
    for g, s, t in cases:
        s = g.src if s is None else s
        t = g.dst if t is None else t
        runs = ((0.0, "src"), (1e-7, "p_asc")) if g.n_edges < 100 else ((1e-9, "src"), (1e-8, "dst"))
        for eps, border in runs:
            a = ctx.reliability(g, s, t, capacity=1 << 22, eps=eps, branch_order=border)
            b = ctx.reliability(g, s, t, capacity=1 << 22, eps=eps, branch_order=border, small_kernel="group")
            assert a.engine == "grid" and a.kernel == "lane" and b.kernel == ""
            for f in ("R", "esp", "nodes", "leaves", "dead_ends", "truncated", "spilled", "paths", "iterations",
                      "max_queue_items"):
                assert getattr(a, f) == getattr(b, f), (g.n_nodes, eps, border, f)
            o = oracle.run(g, s, t, eps=eps, branch_order=border, threads=8)
            assert (a.nodes, a.leaves, a.dead_ends, a.truncated, a.iterations, a.max_queue_items) == \
                (o.nodes, o.leaves, o.dead, o.truncated, o.waves, o.max_wave)
            assert a.R == o.R and a.esp == o.esp
