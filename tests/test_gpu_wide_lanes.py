"""The bucketed whole-GPU queue with one lane per subproblem (nr_bucket_wide_kernel's LANES
instantiation, nr_wide_lane_step): undirected simple graphs of <= 250 nodes, two-terminal path
branching, the src-side-first order.  Every field -- waves, widest wave, counts, queue, stop,
exact R and ESP -- equals the warp-per-subproblem kernel's (small_kernel="group") and the
oracle's; runs that fill the arena spill different records and are brackets of the same value."""
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("R", "esp", "nodes", "leaves", "dead_ends", "truncated", "spilled", "paths", "iterations",
          "max_queue_items", "queued", "stop")


@pytest.fixture(scope="module")
def ctx(engine_lib):
    c = engine_lib.Context(0)
    yield c
    c.close()


CASES = [
    ("rgg 200/600 budget 200K", lambda G: G.rgg(200, 600, p_range=(0.9, 0.99), seed=7), 1e-5, 200_000, 0.0),
    ("rgg 120/300 budget 300K", lambda G: G.rgg(120, 300, p_range=(0.9, 0.99), seed=5), 1e-6, 300_000, 0.0),
    ("rgg 150/400 eps 1e-9 budget 100K", lambda G: G.rgg(150, 400, p_range=(0.85, 0.99), seed=4), 1e-7, 100_000, 1e-9),
    ("grid 10x10 to 1e-4", lambda G: G.grid(10, 10, p_range=(0.9, 0.99), seed=3), 1e-4, 300_000, 0.0),
    ("gnm 40/52 exhaustive", lambda G: G.gnm(40, 52, p_range=(0.5, 0.95), seed=9), 0.0, 0, 0.0),
    ("K40 budget 50K", lambda G: G.complete(40, p_range=(0.6, 0.9), seed=2), 1e-9, 50_000, 0.0),
]


@pytest.mark.parametrize("name,make,target,budget,eps", CASES, ids=[c[0] for c in CASES])
def test_lane_bucket_queue_matches_warp_and_oracle(ctx, oracle, name, make, target, budget, eps):
    from relaibilitygpu_gb300 import graphs
    g = make(graphs)
    s, t = (g.src, g.dst) if g.src != g.dst else (0, g.n_nodes - 1)
    if name.startswith("grid") or name.startswith("K40"):
        s, t = 0, g.n_nodes - 1
    opts = dict(capacity=1 << 23, target_width=target, order="maxmass", bucket_shift=2, n_buckets=255,
                max_nodes=budget, eps=eps, timeout_ms=120000.0)
    a = ctx.reliability(g, s, t, **opts)
    b = ctx.reliability(g, s, t, small_kernel="group", **opts)
    assert a.engine == "grid" and a.kernel == "lane" and b.kernel == "", (a.kernel, b.kernel)
    for f in FIELDS:
        assert getattr(a, f) == getattr(b, f), (f, getattr(a, f), getattr(b, f))
    o = oracle.run(g, s, t, target_width=target, bucket_shift=2, n_buckets=255, max_nodes=budget, eps=eps,
                   threads=8)
    assert (a.nodes, a.leaves, a.dead_ends, a.truncated, a.iterations, a.max_queue_items, a.queued) == \
        (o.nodes, o.leaves, o.dead, o.truncated, o.waves, o.max_wave, o.queued)
    assert a.R == o.R and a.esp == o.esp


def test_lane_bucket_queue_spill_brackets(ctx, oracle):
    """An arena too small for the run: the children past it spill into ESP; both kernels'
    brackets hold the exact value."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.gnm(40, 52, p_range=(0.5, 0.95), seed=9)
    exact = oracle.run(g, g.src, g.dst, threads=8)
    for kernel in ("auto", "group"):
        r = ctx.reliability(g, g.src, g.dst, capacity=3000, order="maxmass", bucket_shift=2, n_buckets=255,
                            small_kernel=kernel)
        assert r.spilled > 0
        assert r.R <= exact.R + 1e-15 and exact.R <= r.R + r.esp + 1e-12


def test_lane_bucket_queue_not_for_other_orders(ctx):
    """Branch orders other than the reference's, fork branching and directed graphs keep the warp
    per subproblem."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.rgg(80, 200, p_range=(0.9, 0.99), seed=1)
    kw = dict(capacity=1 << 20, target_width=1e-4, order="maxmass", bucket_shift=2, n_buckets=255)
    assert ctx.reliability(g, g.src, g.dst, **kw).kernel == "lane"
    assert ctx.reliability(g, g.src, g.dst, branch_order="p_asc", **kw).kernel == ""
    assert ctx.reliability(g, g.src, g.dst, branching="fork", **kw).kernel == ""
