"""Branch orders (NR_BORDER_*: src side first, dst side first, ascending / descending p) on
every engine against the oracle's branch_order, bit for bit: subproblems, waves, widest wave,
queued, R and ESP.  Exhaustive runs also agree with brute force, whatever the order."""
import pytest

from conftest import rel_close

pytestmark = pytest.mark.gpu

ORDERS = ["src", "dst", "p_asc", "p_desc"]


@pytest.fixture(scope="module")
def ctx(engine_lib):
    c = engine_lib.Context(0)
    yield c
    c.close()


def same(r, o):
    assert (r.nodes, r.leaves, r.dead_ends, r.iterations, r.queued) == (o.nodes, o.leaves, o.dead, o.waves, o.queued)
    assert r.R == o.R and r.esp == o.esp, (r.R, o.R, r.esp, o.esp)


@pytest.mark.parametrize("border", ORDERS)
def test_whole_gpu_small_exhaustive(ctx, oracle, border):
    """nr_grid_kernel (n <= 32, breadth-first waves, exhaustive) and brute force."""
    from relaibilitygpu_gb300 import graphs
    for g, s, t in [(graphs.grid(4, 4, p_range=(0.6, 0.95), seed=3), 0, 15),
                    (graphs.complete(8, p_range=(0.5, 0.95), seed=4), 0, 7),
                    (graphs.grid(3, 6, p_range=(0.7, 0.95), seed=5), 0, 17)]:
        r = ctx.reliability(g, s, t, capacity=1 << 22, branch_order=border)
        o = oracle.run(g, s, t, branch_order=border)
        assert r.engine == "grid"
        assert (r.nodes, r.leaves, r.dead_ends, r.iterations, r.max_queue_items) == \
            (o.nodes, o.leaves, o.dead, o.waves, o.max_wave)
        assert r.R == o.R
        if g.n_edges <= 24:
            assert rel_close(r.R, oracle.brute(g, s, t), 1e-12)


@pytest.mark.parametrize("border", ORDERS)
@pytest.mark.parametrize("kernel,shift", [("auto", -1), ("lane1", -1), ("auto", 1), ("group", 1), ("group", -1)])
def test_warp_engine_batches(ctx, oracle, border, kernel, shift):
    """The lane kernels (<= 16 nodes) and the lane-group kernel, one and several buckets; the
    instances' queues fit a warp's pages, so the runs are the oracle's."""
    from relaibilitygpu_gb300 import graphs
    gs = ([graphs.grid(4, 4, p_range=(0.9, 0.99), seed=s) for s in range(12)] +
          [graphs.complete(9, p_range=(0.7, 0.95), seed=s) for s in range(12)] +
          [graphs.complete(20, p_range=(0.9, 0.99), seed=s) for s in range(8)])
    srcs = [0] * len(gs)
    dsts = [g.n_nodes - 1 for g in gs]
    nb = 64 if shift >= 0 else 1
    res = ctx.reliability_batch(gs, srcs, dsts, target_width=1e-4, bucket_shift=shift, n_buckets=64,
                                order="maxmass" if shift >= 0 else "waves", small_kernel=kernel, branch_order=border,
                                pages_per_warp=512)
    compared = 0
    for g, s, t, r in zip(gs, srcs, dsts, res):
        if r.spilled:
            continue
        o = oracle.run(g, s, t, target_width=1e-4, bucket_shift=shift, n_buckets=nb, branch_order=border)
        same(r, o)
        compared += 1
    assert compared >= 28


@pytest.mark.parametrize("border", ORDERS)
@pytest.mark.parametrize("shift", [-1, 2])
def test_wide_engines(ctx, oracle, border, shift):
    """The whole-GPU engines for n > 32: breadth-first waves and the bucketed queue."""
    from relaibilitygpu_gb300 import graphs
    for g, s, t, tw in [(graphs.grid(6, 6, p_range=(0.85, 0.99), seed=2), 0, 35, 1e-4),
                        (lambda x: (x, x.src, x.dst, 1e-3))(graphs.rgg(60, 150, p_range=(0.9, 0.99), seed=1))]:
        nb = 64 if shift >= 0 else 1
        r = ctx.reliability(g, s, t, capacity=1 << 24, target_width=tw, bucket_shift=shift, n_buckets=64,
                            order="maxmass" if shift >= 0 else "waves", branch_order=border, max_nodes=2_000_000)
        o = oracle.run(g, s, t, target_width=tw, bucket_shift=shift, n_buckets=nb, branch_order=border,
                       max_nodes=2_000_000, threads=4)
        assert r.engine == "grid" and r.spilled == 0      # the queue holds every child: the oracle's run
        same(r, o)


def test_noalloc_branch_order(engine_lib, oracle):
    from relaibilitygpu_gb300 import graphs
    g = graphs.grid(4, 4, p_range=(0.6, 0.95), seed=9)
    for border in ORDERS:
        r = engine_lib.reliability_noalloc(g, 0, 15, branch_order=border)
        o = oracle.run(g, 0, 15, branch_order=border)
        assert (r.nodes, r.leaves, r.dead_ends) == (o.nodes, o.leaves, o.dead) and r.R == o.R


def test_branch_order_rejected_where_unsupported(ctx, engine_lib):
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(8, p=0.5)
    with pytest.raises(engine_lib.NrError) as e:
        ctx.reliability(g, 0, 7, branch_order=7)
    assert e.value.status == -1
    with pytest.raises(engine_lib.NrError) as e:
        ctx.reliability_kterminal(graphs.complete(40, p=0.5), [0, 5, 39], branch_order="p_asc")
    assert e.value.status == -4
