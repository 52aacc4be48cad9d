"""Whole-GPU engine for 33..1024 nodes (nr_wide.cuh) against the oracle.

Same bars as the small engines: counts, waves and widest wave bit-exact; R and
ESP (exact fixed-point sums) equal to the oracle's."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(engine_lib):
    c = engine_lib.Context(0)
    yield c
    c.close()


def check(r, o):
    assert (r.paths, r.nodes, r.leaves, r.dead_ends, r.truncated, r.spilled) == \
        (o.paths, o.nodes, o.leaves, o.dead, o.truncated, o.spilled)
    assert (r.iterations, r.max_queue_items) == (o.waves, o.max_wave)
    assert r.R == o.R, (r.R, o.R)
    assert r.esp == o.esp, (r.esp, o.esp)


CASES = [
    ("K40 p=0.5", lambda G: (G.complete(40, p=0.5), 0, 39), 1e-5),
    ("K40 p=0.1 (COMP40)", lambda G: (G.complete(40, p=0.1), 0, 39), 1e-4),
    ("K40 p~U[0.9,0.99]", lambda G: (G.complete(40, p_range=(0.9, 0.99), seed=1), 0, 39), 1e-10),
    ("rgg 200/600", lambda G: (lambda g: (g, g.src, g.dst))(G.rgg(200, 600, p_range=(0.9, 0.99), seed=7)), 1e-5),
    ("rgg 100/250", lambda G: (lambda g: (g, g.src, g.dst))(G.rgg(100, 250, p_range=(0.9, 0.99), seed=3)), 1e-6),
    ("gnm 50/120", lambda G: (lambda g: (g, g.src, g.dst))(G.gnm(50, 120, p_range=(0.5, 0.95), seed=4)), 1e-9),
    ("grid 6x7", lambda G: (G.grid(6, 7, p_range=(0.8, 0.99), seed=2), 0, 41), 1e-7),
    ("gnm 300/1000", lambda G: (lambda g: (g, g.src, g.dst))(G.gnm(300, 1000, p_range=(0.85, 0.99), seed=9)), 1e-5),
    ("path 1000", lambda G: (G.from_edges(1000, [(i, i + 1) for i in range(999)], [0.999] * 999), 0, 999), 0.0),
]


@pytest.mark.parametrize("name,make,eps", CASES, ids=[c[0] for c in CASES])
def test_wide_matches_oracle(ctx, oracle, name, make, eps):
    from relaibilitygpu_gb300 import graphs
    g, s, t = make(graphs)
    o = oracle.run(g, s, t, eps=eps, max_nodes=20_000_000)
    assert o.status == 0
    r = ctx.reliability(g, s, t, capacity=1 << 22, eps=eps)
    assert r.engine == "grid"
    check(r, o)


def test_wide_long_path_exact():
    """A 999-hop path: no 32-node cap (the reference truncates at 32, main.cu:152)."""
    import relaibilitygpu_gb300 as nr
    g = nr.from_edges(1000, [(i, i + 1) for i in range(999)], [0.999] * 999)
    r = nr.reliability(g, 0, 999)
    prod = 1.0
    for _ in range(999):
        prod *= 0.999
    assert r.R == prod and r.paths == 1 and r.nodes == 1000 and r.dead_ends == 999


def test_wide_overflow_brackets(ctx, oracle):
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(40, p=0.5)
    exact = oracle.run(g, 0, 39, eps=1e-6)
    r = ctx.reliability(g, 0, 39, capacity=500, eps=1e-6)
    assert r.spilled > 0
    assert r.R <= exact.R + 1e-15 and exact.R + exact.esp <= r.R + r.esp + 1e-12


def test_wide_limits(ctx, engine_lib, oracle):
    """Masks above 16 blocks (K47: 1081 edges, 68 words) run in the runtime-width instantiation,
    bit for bit against the oracle; graphs above 16384 nodes are refused."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(47, p=0.5)
    for shift, nb in ((2, 255), (-1, 1)):
        r = ctx.reliability(g, 0, 46, capacity=1 << 22, target_width=1e-2, bucket_shift=shift, n_buckets=255,
                            order="maxmass" if shift >= 0 else "waves", max_nodes=20000)
        o = oracle.run(g, 0, 46, target_width=1e-2, bucket_shift=shift, n_buckets=nb, max_nodes=20000, threads=8)
        assert r.engine == "grid" and r.spilled == 0
        check(r, o)
    n = 16385
    big = graphs.from_edges(n, [(i, i + 1) for i in range(n - 1)], [0.99] * (n - 1))
    with pytest.raises(engine_lib.NrError) as e:
        ctx.reliability(big, 0, n - 1)
    assert e.value.status == -4


TARGET_CASES = [
    ("rgg 200/600 to 1e-2", lambda G: (lambda g: (g, g.src, g.dst))(G.rgg(200, 600, p_range=(0.9, 0.99), seed=7)),
     1e-2),
    ("rgg 100/250 to 1e-3", lambda G: (lambda g: (g, g.src, g.dst))(G.rgg(100, 250, p_range=(0.9, 0.99), seed=3)),
     1e-3),
    ("rgg 60/150 to 1e-6", lambda G: (lambda g: (g, g.src, g.dst))(G.rgg(60, 150, p_range=(0.9, 0.99), seed=11)),
     1e-6),
    ("K40 p~U[0.9,0.99] to 1e-9", lambda G: (G.complete(40, p_range=(0.9, 0.99), seed=1), 0, 39), 1e-9),
    ("grid 6x6 to 1e-3", lambda G: (G.grid(6, 6, p_range=(0.8, 0.99), seed=5), 0, 35), 1e-3),
    ("target above 1: root only", lambda G: (G.complete(40, p=0.5), 0, 39), 2.0),
]


@pytest.mark.parametrize("name,make,target", TARGET_CASES, ids=[c[0] for c in TARGET_CASES])
def test_wide_target_width_matches_oracle(ctx, oracle, name, make, target):
    """Truncated runs: breadth-first waves stopped once ESP + queued mass <= target, as the
    oracle's wave schedule with one bucket -- same waves, counts, queue and exact sums."""
    from relaibilitygpu_gb300 import graphs
    g, s, t = make(graphs)
    o = oracle.run(g, s, t, target_width=target, threads=4)
    assert o.status in (0, 1)
    r = ctx.reliability(g, s, t, capacity=1 << 23, target_width=target, bucket_shift=-1)
    assert r.engine == "grid"
    check(r, o)
    assert (r.queued, r.stop) == (o.queued, o.status)
    assert r.esp <= target or o.status == 0


def test_batch_routes_large_graphs_to_wide_engine(ctx, oracle):
    """Batches mix graphs above 32 nodes (whole-GPU engine, side by side) with small ones
    (warp engine, all together); with one bucket both follow the oracle's wave schedule."""
    from relaibilitygpu_gb300 import graphs
    gs = []
    for i in range(24):
        if i % 6 == 0:
            gs.append(graphs.grid(6, 6, p_range=(0.8, 0.99), seed=60 + i))
        elif i % 6 == 3:
            gs.append(graphs.rgg(60, 150, p_range=(0.9, 0.99), seed=60 + i))
        else:
            gs.append(graphs.gnm(8 + i % 12, 20 + i, p_range=(0.8, 0.99), seed=60 + i))
    res = ctx.reliability_batch(gs, [g.src for g in gs], [g.dst for g in gs], capacity=1 << 16,
                                target_width=1e-3, bucket_shift=-1)
    for g, r in zip(gs, res):
        o = oracle.run(g, g.src, g.dst, target_width=1e-3)
        assert r.engine == ("grid" if g.n_nodes > 32 else "warp")
        assert (r.n_nodes, r.src, r.dst) == (g.n_nodes, g.src, g.dst)
        check(r, o)
        assert r.queued == o.queued


def test_batch_runs_large_graphs_side_by_side(ctx, oracle):
    """A batch's graphs above 32 nodes (breadth-first waves) share cooperative launches, each on
    its own group of blocks with its own waves, barrier and stop tests: every field equals the
    one-at-a-time run's, for compiled and runtime mask widths, budgets and eps truncation."""
    from relaibilitygpu_gb300 import graphs
    gs = ([graphs.grid(6, 6, p_range=(0.8, 0.99), seed=80 + s) for s in range(4)] +
          [graphs.grid(6, 7, p_range=(0.85, 0.99), seed=85), graphs.rgg(60, 150, p_range=(0.9, 0.99), seed=86),
           graphs.rgg(60, 150, p_range=(0.9, 0.99), seed=87), graphs.rgg(100, 300, p_range=(0.9, 0.99), seed=88),
           graphs.complete(40, p_range=(0.9, 0.99), seed=89), graphs.complete(50, p_range=(0.95, 0.99), seed=90)])
    srcs = [g.src if g.n_nodes not in (40, 50) else 0 for g in gs]
    dsts = [g.dst if g.n_nodes not in (40, 50) else g.n_nodes - 1 for g in gs]
    fields = ("R", "esp", "nodes", "leaves", "dead_ends", "truncated", "spilled", "paths", "iterations",
              "max_queue_items", "queued", "stop")
    compared = 0
    for opts in (dict(target_width=1e-3), dict(target_width=1e-7, max_nodes=20000), dict(eps=1e-9, target_width=1e-3)):
        res = ctx.reliability_batch(gs, srcs, dsts, capacity=1 << 22, bucket_shift=-1, **opts)
        for k, (g, s, t, r) in enumerate(zip(gs, srcs, dsts, res)):
            one = ctx.reliability(g, s, t, capacity=1 << 22, bucket_shift=-1, **opts)
            assert r.engine == "grid" and one.engine == "grid"
            if r.spilled or one.spilled:      # which records a full buffer spills depends on the
                assert max(r.R, one.R) <= min(r.R + r.esp, one.R + one.esp) + 1e-15   # launch: brackets
                continue
            compared += 1
            for f in fields:
                assert getattr(r, f) == getattr(one, f), (k, opts, f, getattr(r, f), getattr(one, f))
            if k % 3 == 0:
                o = oracle.run(g, s, t, target_width=opts["target_width"], max_nodes=opts.get("max_nodes", 0),
                               eps=opts.get("eps", 0.0), threads=4)
                check(r, o)
                assert r.queued == o.queued
    assert compared >= 24


def test_batch_large_graph_learned_order_unsupported(ctx, engine_lib):
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(8, p=0.9), graphs.grid(6, 6, p=0.9)]
    with pytest.raises(engine_lib.NrError) as e:
        ctx.reliability_batch(gs, [0, 0], [7, 35], target_width=1e-6, order="learned")
    assert e.value.status in (-1, -4)


BUCKET_CASES = [
    ("K40 p~U[0.9,0.99] to 1e-9", lambda G: (G.complete(40, p_range=(0.9, 0.99), seed=1), 0, 39), 1e-9, 2, 1 << 20),
    ("rgg 60/150 to 1e-7", lambda G: (lambda g: (g, g.src, g.dst))(G.rgg(60, 150, p_range=(0.9, 0.99), seed=11)),
     1e-7, 2, 1 << 22),
    ("rgg 100/250 to 1e-4", lambda G: (lambda g: (g, g.src, g.dst))(G.rgg(100, 250, p_range=(0.9, 0.99), seed=3)),
     1e-4, 2, 1 << 24),
    ("gnm 40/52 exhaustive", lambda G: (lambda g: (g, g.src, g.dst))(G.gnm(40, 52, p_range=(0.5, 0.95), seed=9)),
     0.0, 2, 1 << 20),
    ("gnm 36/45 exhaustive, one bucket per octave", lambda G: (lambda g: (g, g.src, g.dst))(
        G.gnm(36, 45, p_range=(0.5, 0.95), seed=8)), 0.0, 0, 1 << 20),
]


@pytest.mark.parametrize("name,make,target,shift,cap", BUCKET_CASES, ids=[c[0] for c in BUCKET_CASES])
def test_bucket_queue_matches_oracle(ctx, oracle, name, make, target, shift, cap):
    """The whole-GPU bucketed max-mass queue: each wave is the whole highest bucket, as the
    oracle's bucketed wave schedule -- same waves, widest wave, counts, queue and exact sums."""
    from relaibilitygpu_gb300 import graphs
    g, s, t = make(graphs)
    o = oracle.run(g, s, t, target_width=target, bucket_shift=shift, n_buckets=255, threads=4)
    assert o.status in (0, 1)
    r = ctx.reliability(g, s, t, capacity=cap, target_width=target, order="maxmass", bucket_shift=shift,
                        n_buckets=255)
    assert r.engine == "grid"
    check(r, o)
    assert (r.queued, r.stop) == (o.queued, o.status)


def test_bucket_queue_reclaims_freed_slots(ctx, oracle):
    """2.09M records are pushed over the run, at most 1.38M at a time: an arena of 1.8M slots
    holds the run only if the slots of popped records are reused (no spill, exact match)."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.rgg(60, 150, p_range=(0.9, 0.99), seed=11)
    o = oracle.run(g, g.src, g.dst, target_width=1e-7, bucket_shift=2, n_buckets=255, threads=4)
    assert o.pushes > 1_800_000 > o.max_queued
    r = ctx.reliability(g, g.src, g.dst, capacity=1_800_000, target_width=1e-7, order="maxmass", bucket_shift=2,
                        n_buckets=255)
    assert r.spilled == 0
    check(r, o)


def test_bucket_queue_overflow_brackets(ctx, oracle):
    """A full arena spills children into ESP: R <= true <= R + ESP still holds."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.gnm(40, 52, p_range=(0.5, 0.95), seed=9)
    exact = oracle.run(g, g.src, g.dst)
    r = ctx.reliability(g, g.src, g.dst, capacity=2000, order="maxmass", bucket_shift=2, n_buckets=255)
    assert r.spilled > 0
    assert r.R <= exact.R + 1e-15 and exact.R <= r.R + r.esp + 1e-12


def test_bucket_queue_node_budget(ctx, oracle):
    """A node budget stops between waves with a valid bracket (stop reason 3)."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.rgg(100, 250, p_range=(0.9, 0.99), seed=3)
    r = ctx.reliability(g, g.src, g.dst, capacity=1 << 23, target_width=1e-9, order="maxmass", bucket_shift=2,
                        n_buckets=255, max_nodes=200_000)
    assert r.stop == 3 and r.nodes >= 200_000
    o = oracle.run(g, g.src, g.dst, target_width=1e-9, bucket_shift=2, n_buckets=255, threads=4,
                   max_nodes=200_000)
    check(r, o)


def test_checkpoint_resume_continues_the_same_run(ctx, engine_lib, tmp_path):
    """A bucketed run stopped at a node budget, saved and resumed (twice) ends exactly where the
    uninterrupted run ends: same waves, counts, queue and exact sums."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.rgg(60, 150, p_range=(0.9, 0.99), seed=11)
    opts = dict(order="maxmass", bucket_shift=2, n_buckets=255, target_width=1e-7)
    full = ctx.reliability(g, g.src, g.dst, capacity=1 << 22, **opts)
    assert full.stop == 1
    part = ctx.reliability(g, g.src, g.dst, capacity=1 << 22, max_nodes=150_000, **opts)
    assert part.stop == 3 and part.nodes < full.nodes
    p1 = str(tmp_path / "a.ckpt")
    ctx.checkpoint_save(p1)
    mid = ctx.checkpoint_resume(p1, g, g.src, g.dst, capacity=1 << 22, max_nodes=400_000, **opts)
    assert mid.stop == 3 and part.nodes < mid.nodes < full.nodes
    p2 = str(tmp_path / "b.ckpt")
    ctx.checkpoint_save(p2)
    end = ctx.checkpoint_resume(p2, g, g.src, g.dst, capacity=1 << 22, **opts)
    for f in ("R", "esp", "nodes", "leaves", "dead_ends", "paths", "iterations", "max_queue_items", "queued", "stop"):
        assert getattr(end, f) == getattr(full, f), f
    # another graph, or other buckets, cannot resume this file
    other = graphs.rgg(60, 150, p_range=(0.9, 0.99), seed=12)
    with pytest.raises(engine_lib.NrError) as e:
        ctx.checkpoint_resume(p2, other, other.src, other.dst, **opts)
    assert e.value.status == -1
    with pytest.raises(engine_lib.NrError):
        ctx.checkpoint_resume(p2, g, g.src, g.dst, **dict(opts, bucket_shift=1))
    # a run on another engine invalidates the saved state
    ctx.reliability(graphs.complete(40, p=0.5), 0, 39, capacity=1 << 16, eps=1e-3)
    with pytest.raises(engine_lib.NrError):
        ctx.checkpoint_save(str(tmp_path / "c.ckpt"))


KT_CASES = [
    ("K7 3 terminals", lambda G: G.complete(7, p_range=(0.5, 0.95), seed=2), [0, 3, 6]),
    ("grid 3x4 4 terminals", lambda G: G.grid(3, 4, p_range=(0.6, 0.97), seed=4), [0, 5, 11, 3]),
    ("gnm 9/15 root 2", lambda G: G.gnm(9, 15, p_range=(0.4, 0.95), seed=6), [2, 0, 8, 4, 7]),
    ("directed 4-cycle", lambda G: G.from_arcs(4, [(0, 1), (1, 2), (2, 3), (3, 0), (0, 2)],
                                               [0.9, 0.8, 0.7, 0.6, 0.5]), [0, 2, 3]),
    ("repeated terminals", lambda G: G.grid(3, 3, p_range=(0.6, 0.97), seed=1), [4, 0, 8, 0, 8]),
]


@pytest.mark.parametrize("name,make,term", KT_CASES, ids=[c[0] for c in KT_CASES])
def test_k_terminal_exact(ctx, oracle, name, make, term):
    """K-terminal reliability (every terminal joined to terminals[0]) on the whole-GPU engine:
    the oracle's waves, counts and exact sums, and brute force over the edge states."""
    from relaibilitygpu_gb300 import graphs
    g = make(graphs)
    exact = oracle.brute_k(g, term)
    o = oracle.run(g, 0, 0, terminals=term)
    assert o.status == 0
    r = ctx.reliability_kterminal(g, term, capacity=1 << 20)
    assert r.engine == "grid" and (r.src, r.dst) == (term[0], term[-1])
    check(r, o)
    assert abs(r.R - exact) <= 1e-13


KT_WIDE_CASES = [
    ("K40 p=0.5, 4 terminals", lambda G: G.complete(40, p=0.5), [0, 13, 27, 39], dict(eps=1e-4)),
    ("grid 6x7 corners", lambda G: G.grid(6, 7, p_range=(0.8, 0.99), seed=2), [0, 6, 35, 41], dict(eps=1e-7)),
    ("rgg 100/250 to 1e-3, waves", lambda G: G.rgg(100, 250, p_range=(0.9, 0.99), seed=3), [0, 17, 55, 99],
     dict(target_width=1e-3, bucket_shift=-1)),
    ("rgg 60/150 to 1e-5, buckets", lambda G: G.rgg(60, 150, p_range=(0.9, 0.99), seed=11), [5, 20, 40, 59],
     dict(target_width=1e-5, bucket_shift=2, n_buckets=255)),
    ("gnm 40/52 exhaustive, buckets", lambda G: G.gnm(40, 52, p_range=(0.5, 0.95), seed=9), [0, 9, 19, 29, 39],
     dict(bucket_shift=1, n_buckets=255, order="maxmass")),
]


@pytest.mark.parametrize("name,make,term,kw", KT_WIDE_CASES, ids=[c[0] for c in KT_WIDE_CASES])
def test_k_terminal_matches_oracle(ctx, oracle, name, make, term, kw):
    """Larger K-terminal runs, truncated (eps), target-stopped (waves or buckets) or exhaustive:
    the same schedule, counts, queue and exact sums as the oracle."""
    from relaibilitygpu_gb300 import graphs
    g = make(graphs)
    okw = {k: v for k, v in kw.items() if k != "order"}
    o = oracle.run(g, 0, 0, terminals=term, threads=4, max_nodes=20_000_000, **okw)
    assert o.status in (0, 1)
    r = ctx.reliability_kterminal(g, term, capacity=1 << 22, **kw)
    check(r, o)
    assert (r.queued, r.stop) == (o.queued, o.status)


def test_k_terminal_two_terminals_is_the_two_terminal_run(ctx, engine_lib):
    """terminals [s, t] is the two-terminal problem on the same engine, bit for bit; terminals
    [s] alone gives R = 1; fork branching and the learned order are refused."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.rgg(60, 150, p_range=(0.9, 0.99), seed=11)
    for kw in (dict(eps=1e-6), dict(target_width=1e-6, bucket_shift=2, n_buckets=255, order="maxmass")):
        a = ctx.reliability(g, g.src, g.dst, capacity=1 << 22, **kw)
        b = ctx.reliability_kterminal(g, [g.src, g.dst], capacity=1 << 22, **kw)
        for f in ("R", "esp", "nodes", "leaves", "dead_ends", "paths", "iterations", "max_queue_items", "queued"):
            assert getattr(a, f) == getattr(b, f), (kw, f)
    one = ctx.reliability_kterminal(g, [7])
    assert one.R == 1.0 and one.esp == 0.0
    for bad in (dict(branching="fork"), dict(order="learned")):
        with pytest.raises(engine_lib.NrError) as e:
            ctx.reliability_kterminal(g, [0, 5, 9], **bad)
        assert e.value.status in (-1, -4)
    with pytest.raises(engine_lib.NrError):
        ctx.reliability_kterminal(g, [0, 60])


@pytest.mark.parametrize("shift", [2, -1])
def test_directed_graph_beyond_1024_nodes(ctx, oracle, shift):
    """A directed graph of the size class of the reference's directed example (workingPad's
    6301-node, 20,777-arc peer-to-peer overlay: out-degree <= 10, p = 0.5): more than 1024 nodes
    and a 1299-word mask, so the runtime-width kernels with the graph tables in global memory.
    Bit for bit against the oracle at a budget, bucketed queue and breadth-first waves."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.random_digraph(6301, 20777, p=0.5, seed=1)
    budget, nb = (3000, 255) if shift >= 0 else (500, 1)
    r = ctx.reliability(g, g.src, g.dst, capacity=(1 << 20) if shift >= 0 else (1 << 16), target_width=1e-3,
                        order="maxmass" if shift >= 0 else "waves", bucket_shift=shift, n_buckets=255,
                        max_nodes=budget)
    o = oracle.run(g, g.src, g.dst, target_width=1e-3, bucket_shift=shift, n_buckets=nb, max_nodes=budget, threads=8)
    assert r.engine == "grid" and r.spilled == 0 and r.stop == 3
    check(r, o)
