"""nr_reliability_noalloc: the entry point for callers that cannot call cudaMalloc.

Such callers (an application whose device memory belongs to its own allocator
or pool, a plugin that may not grow the process footprint) get the solve done
inside a static device array.  This checks, through the C ABI, that two calls
in a row give the results of the allocating entry point: counts bit-exact and
R, ESP within 1e-12, the tolerance of the other GPU tests; that a run stopped
by its pop budget returns a valid bracket; and that bad input is rejected.
The file is named to be collected last."""
import numpy as np
import pytest

from conftest import rel_close

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert (a.nodes, a.leaves, a.dead_ends, a.truncated, a.spilled, a.paths, a.queued) == \
        (b.nodes, b.leaves, b.dead_ends, b.truncated, b.spilled, b.paths, b.queued)
    if a.engine == b.engine:    # exhaustive runs: waves (whole-GPU engine) vs pages here
        assert a.iterations == b.iterations
    assert rel_close(a.R, b.R, 1e-12)
    assert abs(a.esp - b.esp) <= 1e-12 * max(b.esp, 1e-300) + 1e-18


def _directed(seed):
    from relaibilitygpu_gb300 import graphs
    rng = np.random.default_rng(seed)
    n = 9
    arcs = [(u, v) for u in range(n) for v in range(n) if u != v and rng.random() < 0.45]
    return graphs.from_arcs(n, arcs, rng.uniform(0.6, 0.97, size=len(arcs)))


def test_noalloc_matches_allocating_entry_point(engine_lib):
    from relaibilitygpu_gb300 import graphs
    cases = [
        (graphs.complete(15, p_range=(0.9, 0.99), seed=7), 0, 14, dict(target_width=1e-6)),
        (graphs.complete(8, p=0.5), 0, 7, dict(order="maxmass")),
        (graphs.grid(3, 4, p_range=(0.6, 0.95), seed=2), 0, 11, dict()),
        (_directed(3), 0, 8, dict()),                                    # a 'D' graph: one edge per arc
        (graphs.complete(8, p_range=(0.5, 0.95), seed=4), 0, 7, dict(branching="fork")),
    ]
    with engine_lib.Context(0) as ctx:
        for g, s, t, kw in cases:
            ref = ctx.reliability(g, s, t, capacity=1 << 16, **kw)
            for _ in range(2):                      # two calls in a row share the static array
                got = engine_lib.reliability_noalloc(g, s, t, **kw)
                assert got.spilled == 0
                assert got.stop == ref.stop
                _same(got, ref)


def test_noalloc_budget_stop_is_a_bracket(engine_lib):
    """An exhaustive run past its pop budget stops with stop = 3, the queued mass in ESP."""
    from relaibilitygpu_gb300 import graphs
    g9 = graphs.complete(9, p=0.5)
    g15 = graphs.complete(15, p_range=(0.9, 0.99), seed=11)
    with engine_lib.Context(0) as ctx:
        exact = ctx.reliability(g9, 0, 8).R                     # exhaustive K9 on the whole-GPU engine
        tight = ctx.reliability(g15, 0, 14, target_width=1e-12, capacity=1 << 16)
    for _ in range(2):
        got = engine_lib.reliability_noalloc(g9, 0, 8, max_nodes=20000)
        assert got.stop == 3 and got.nodes >= 20000 and got.queued > 0
        assert got.R <= exact * (1 + 1e-12) and exact <= (got.R + got.esp) * (1 + 1e-12)
    got = engine_lib.reliability_noalloc(g15, 0, 14, max_nodes=3000)
    assert got.stop == 3 and got.nodes >= 3000
    assert got.R <= (tight.R + tight.esp) * (1 + 1e-12)
    assert tight.R <= (got.R + got.esp) * (1 + 1e-12)


def test_noalloc_rejects_bad_input(engine_lib):
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(40, p=0.5)
    with pytest.raises(engine_lib.NrError) as e:
        engine_lib.reliability_noalloc(g, 0, 39)
    assert e.value.status == -4                     # NR_ERR_UNSUPPORTED: above 32 nodes
    g = graphs.complete(6, p=0.5)
    g.edge_p = np.array(g.edge_p, dtype=np.float64)
    g.edge_p[3] = np.nan
    with pytest.raises(engine_lib.NrError) as e:
        engine_lib.reliability_noalloc(g, 0, 5)
    assert e.value.status == -1                     # NR_ERR_INVALID: a NaN probability
