"""nr_reliability_noalloc: the entry point for callers that cannot call cudaMalloc.

Such callers (an application whose device memory belongs to its own allocator
or pool, a plugin that may not grow the process footprint) get the solve done
inside a static device array.  This checks, through the C ABI, that two calls
in a row give the results of the allocating entry point: counts bit-exact and
R, ESP within 1e-12, the tolerance of the other GPU tests.  The file is named
to be collected last."""
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


def test_noalloc_matches_allocating_entry_point(engine_lib):
    from relaibilitygpu_gb300 import graphs
    cases = [
        (graphs.complete(15, p_range=(0.9, 0.99), seed=7), 0, 14, dict(target_width=1e-6)),
        (graphs.complete(8, p=0.5), 0, 7, dict(order="maxmass")),
        (graphs.grid(3, 4, p_range=(0.6, 0.95), seed=2), 0, 11, dict()),
    ]
    with engine_lib.Context(0) as ctx:
        for g, s, t, kw in cases:
            ref = ctx.reliability(g, s, t, capacity=1 << 16, **kw)
            for _ in range(2):                      # two calls in a row share the static array
                got = engine_lib.reliability_noalloc(g, s, t, **kw)
                assert got.spilled == 0
                _same(got, ref)


def test_noalloc_rejects_large_graph(engine_lib):
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(40, p=0.5)
    with pytest.raises(engine_lib.NrError) as e:
        engine_lib.reliability_noalloc(g, 0, 39)
    assert e.value.status == -4
