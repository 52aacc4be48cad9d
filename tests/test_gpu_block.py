"""The block kernel (nr_block_lane.cuh): in breadth-first waves the two-slot lane kernel hands an
instance over at a wave boundary once its next wave holds more than `handover_pages` pages, and
the block kernel runs it again from its root on a block of warps.

The schedule is the lane kernels' (waves, stop tests between them, parent rule, children, FP64
products), so every field -- waves, widest wave, counts, queue, exact R and ESP sums -- equals the
two-slot kernel's without hand-over, the lane-group kernel's and the oracle's.  Only which
children spill when a wave outgrows its buffer can differ: such runs are brackets of the same
value."""
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("R", "esp", "nodes", "leaves", "dead_ends", "truncated", "spilled", "paths", "iterations",
          "max_queue_items", "queued", "stop")


@pytest.fixture(scope="module")
def ctx(engine_lib):
    c = engine_lib.Context(0)
    yield c
    c.close()


def uneven_small(count, seed):
    """The uneven generator's graphs of <= 32 nodes (grids up to 5 x 6 and 6 x 5, G(n,m) up to 20
    nodes): waves from a few records to tens of thousands."""
    from relaibilitygpu_gb300 import graphs
    gs = [g for g in graphs.batch_instances(count, seed=seed) if g.n_nodes <= 32]
    return gs, [g.src for g in gs], [g.dst for g in gs]


def same_or_bracket(a, b, i):
    """Equal fields, or (a wave spilled in one of them) brackets of the same value."""
    if a.spilled or b.spilled:
        assert max(a.R, b.R) <= min(a.R + a.esp, b.R + b.esp) + 1e-15, i
        return False
    for f in FIELDS:
        assert getattr(a, f) == getattr(b, f), (i, f, getattr(a, f), getattr(b, f))
    return True


def test_handover_matches_two_slot_group_and_oracle(ctx, oracle):
    """The uneven mix to ESP width <= 1e-6 or 16,384 subproblems (checked between waves): the
    instances whose waves outgrow 8 pages (the default) run on the block kernel; every field equals the
    two-slot kernel's run without hand-over and the lane-group kernel's; a sample of the
    handed-over instances equals the oracle."""
    gs, srcs, dsts = uneven_small(384, seed=11)
    opts = dict(target_width=1e-6, max_nodes=16384, order="waves", n_buckets=64, pages_per_warp=4096)
    a = ctx.reliability_batch(gs, srcs, dsts, **opts)
    b = ctx.reliability_batch(gs, srcs, dsts, handover_pages=-1, **opts)
    c = ctx.reliability_batch(gs, srcs, dsts, small_kernel="group", **opts)
    kinds = [r.kernel for r in a]
    assert kinds.count("block") >= 50 and kinds.count("lane2") >= 50, (kinds.count("block"), kinds.count("lane2"))
    assert {r.kernel for r in b} == {"lane2"} and {r.kernel for r in c} == {"group"}
    same = 0
    checked = 0
    for i, (g, x, y, z) in enumerate(zip(gs, a, b, c)):
        same += same_or_bracket(x, y, i)
        same_or_bracket(x, z, i)
        if x.kernel == "block" and not x.spilled and checked < 24:
            o = oracle.run(g, srcs[i], dsts[i], target_width=1e-6, max_nodes=16384)
            assert (x.nodes, x.leaves, x.dead_ends, x.iterations, x.max_queue_items, x.queued) == \
                (o.nodes, o.leaves, o.dead, o.waves, o.max_wave, o.queued), i
            assert x.R == o.R and x.esp == o.esp, i
            checked += 1
    assert same >= len(gs) - 16 and checked == 24
    # the part's device time covers both launches
    assert len({r.ms for r in a}) == 1


@pytest.mark.parametrize("eps,border,budget", [(0.0, "src", 0), (1e-9, "p_asc", 0), (0.0, "dst", 3000)])
def test_handover_everywhere(ctx, oracle, eps, border, budget):
    """handover_pages = 1: every instance with a wave above 32 records runs on the block kernel
    (graphs of 9..25 nodes, 16- and 32-bit rows, mask widths 1..5 blocks), with eps truncation,
    branch orders and budgets; fields equal the run without hand-over and the oracle's."""
    from relaibilitygpu_gb300 import graphs
    gs, st = [], []
    for s in range(4):
        gs.append(graphs.complete(9 + s, p_range=(0.7, 0.99), seed=1100 + s)); st.append((0, 8 + s))
        gs.append(graphs.grid(4, 4, p_range=(0.7, 0.99), seed=1110 + s)); st.append((0, 15))
        gs.append(graphs.grid(3, 6, p_range=(0.8, 0.99), seed=1120 + s)); st.append((0, 17))
        g = graphs.gnm(24, 70, p_range=(0.85, 0.99), seed=1130 + s); gs.append(g); st.append((g.src, g.dst))
        gs.append(graphs.complete(20, p_range=(0.9, 0.99), seed=1140 + s)); st.append((0, 19))
    gs.append(graphs.complete(25, p_range=(0.9, 0.99), seed=1150)); st.append((0, 24))
    srcs, dsts = [x for x, _ in st], [y for _, y in st]
    opts = dict(target_width=1e-7, eps=eps, order="waves", n_buckets=64, capacity=1 << 17,
                branch_order=border, max_nodes=budget)
    a = ctx.reliability_batch(gs, srcs, dsts, handover_pages=1, **opts)
    b = ctx.reliability_batch(gs, srcs, dsts, handover_pages=-1, **opts)
    assert sum(r.kernel == "block" for r in a) >= 12
    for i, (g, x, y) in enumerate(zip(gs, a, b)):
        assert x.spilled == 0 and y.spilled == 0, i      # (widest waves: 25K records)
        same_or_bracket(x, y, i)
        if i % 2 == 0:
            o = oracle.run(g, srcs[i], dsts[i], target_width=1e-7, eps=eps, branch_order=border, max_nodes=budget)
            assert (x.nodes, x.leaves, x.dead_ends, x.truncated, x.iterations, x.max_queue_items, x.queued) == \
                (o.nodes, o.leaves, o.dead, o.truncated, o.waves, o.max_wave, o.queued), i
            assert x.R == o.R and x.esp == o.esp, i


def test_single_instance_handover_and_block_spill(ctx, oracle):
    """One instance through nr_reliability: its waves outgrow the warp and the block kernel
    finishes it (the oracle's fields); with a small queue the block kernel's wave buffer fills and
    spills into ESP, and the bracket holds the exact value."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.grid(4, 5, p_range=(0.8, 0.99), seed=1200)      # 139K subproblems, widest wave 81K
    r = ctx.reliability(g, 0, 19, target_width=1e-5, order="waves", n_buckets=64, capacity=1 << 18)
    o = oracle.run(g, 0, 19, target_width=1e-5)
    assert r.kernel == "block" and r.spilled == 0
    assert (r.nodes, r.iterations, r.max_queue_items, r.queued) == (o.nodes, o.waves, o.max_wave, o.queued)
    assert r.R == o.R and r.esp == o.esp
    k9 = graphs.complete(9, p_range=(0.6, 0.97), seed=5)
    exact = oracle.run(k9, 0, 8)
    s = ctx.reliability(k9, 0, 8, target_width=1e-14, order="waves", n_buckets=64, capacity=256, handover_pages=1)
    assert s.kernel == "block" and s.spilled > 0
    assert s.R <= exact.R + 1e-15 and exact.R <= s.R + s.esp + 1e-12


def mid_batch():
    """Undirected simple graphs of 33..64 nodes (mask widths 1..4 blocks) for the 64-bit-row block
    kernel, and edge cases: src == dst, certain edges (p = 0 and 1 in the root's mask), a 64-node
    path (63 BFS levels)."""
    from relaibilitygpu_gb300 import graphs
    gs, st = [], []
    for s in range(16):
        gs.append(graphs.grid(6, 6, p_range=(0.8, 0.99), seed=1300 + s)); st.append((0, 35))
    for s in range(8):
        gs.append(graphs.grid(7, 7, p_range=(0.85, 0.99), seed=1320 + s)); st.append((0, 48))
        g = graphs.gnm(40, 100, p_range=(0.8, 0.99), seed=1330 + s); gs.append(g); st.append((g.src, g.dst))
        g = graphs.gnm(60, 180, p_range=(0.85, 0.99), seed=1340 + s); gs.append(g); st.append((g.src, g.dst))
    for s in range(4):
        g = graphs.gnm(64, 250, p_range=(0.9, 0.99), seed=1350 + s); gs.append(g); st.append((g.src, g.dst))
    g = graphs.grid(6, 6, p_range=(0.8, 0.99), seed=1360)
    p = g.edge_p.copy(); p[2] = 0.0; p[5] = 1.0; p[17] = 0.0
    gs.append(graphs.from_edges(36, g.edge_list(), p)); st.append((0, 35))
    gs.append(graphs.grid(6, 6, p_range=(0.8, 0.99), seed=1361)); st.append((14, 14))
    gs.append(graphs.from_edges(64, [(i, i + 1) for i in range(63)], [0.99] * 63)); st.append((0, 63))
    return gs, [a for a, _ in st], [b for _, b in st]


@pytest.mark.parametrize("target,budget,border", [(1e-6, 20000, "src"), (1e-5, 100000, "p_asc"), (1e-6, 5000, "dst")])
def test_mid_graphs_block_kernel(ctx, oracle, target, budget, border):
    """A batch's graphs of 33..64 nodes in breadth-first waves run one block each with 64-bit rows
    rebuilt from the mask; every field equals the whole-GPU wide engine's (small_kernel="group"
    keeps them there) and the oracle's.  A 2^22-record capacity holds every wave (the widest, the
    children of the last wave before a 100 K budget, exceed the default 2^20 a block)."""
    gs, srcs, dsts = mid_batch()
    opts = dict(target_width=target, max_nodes=budget, order="waves", n_buckets=64, branch_order=border,
                capacity=1 << 22)
    a = ctx.reliability_batch(gs, srcs, dsts, **opts)
    b = ctx.reliability_batch(gs, srcs, dsts, small_kernel="group", **opts)
    assert {r.kernel for r in a} == {"block"} and {r.engine for r in b} == {"grid"}
    checked = 0
    for i, (g, x, y) in enumerate(zip(gs, a, b)):
        assert x.spilled == 0 and y.spilled == 0, i
        same_or_bracket(x, y, i)
        if i % 3 == 0 or i >= len(gs) - 3:
            o = oracle.run(g, srcs[i], dsts[i], target_width=target, max_nodes=budget, branch_order=border)
            assert (x.nodes, x.leaves, x.dead_ends, x.iterations, x.max_queue_items, x.queued) == \
                (o.nodes, o.leaves, o.dead, o.waves, o.max_wave, o.queued), i
            assert x.R == o.R and x.esp == o.esp, i
            assert x.stop == {0: 0, 1: 1, 2: 3}[o.status], i      # (the oracle's 2 is the budget)
            checked += 1
    assert checked >= 16


def test_matrix_batches_hand_over(ctx, engine_lib, oracle):
    """One 5 x 5 grid topology with 256 probability rows through the matrix entry points
    (synchronous and submitted): the instances whose waves outgrow the warp run on the block
    kernel from their own row; every field equals the per-instance batch's, the run without
    hand-over and (a sample) the oracle's."""
    import numpy as np
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.grid(5, 5, p_range=(0.8, 0.99), seed=1400 + s) for s in range(256)]
    pm = np.stack([g.edge_p for g in gs])
    opts = dict(target_width=1e-6, max_nodes=16384, order="waves", n_buckets=64, pages_per_warp=4096)
    mb = engine_lib.MatrixBatch(gs[0], pm, 0, 24)
    a = ctx.run_matrix(mb, **opts)
    b = ctx.run_matrix(mb, handover_pages=-1, **opts)
    c = ctx.reliability_batch(gs, [0] * len(gs), [24] * len(gs), **opts)
    t = ctx.submit_matrix(mb, **opts)
    ctx.wait(t)
    d = [engine_lib.Result.from_raw(mb.res[i]) for i in range(len(gs))]
    assert sum(r.kernel == "block" for r in a) >= 32 and {r.kernel for r in b} == {"lane2"}
    for i in range(len(gs)):
        same_or_bracket(a[i], b[i], i)
        same_or_bracket(a[i], c[i], i)
        same_or_bracket(a[i], d[i], i)
        assert a[i].kernel == c[i].kernel == d[i].kernel, i
        if i % 16 == 0 and not a[i].spilled:
            o = oracle.run(gs[i], 0, 24, target_width=1e-6, max_nodes=16384)
            assert (a[i].nodes, a[i].iterations, a[i].max_queue_items, a[i].queued) == \
                (o.nodes, o.waves, o.max_wave, o.queued), i
            assert a[i].R == o.R and a[i].esp == o.esp, i
