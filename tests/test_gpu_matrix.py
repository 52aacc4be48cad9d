"""One topology with a matrix of probability sets (nr_batch_submit_matrix /
nr_reliability_batch_matrix) against the per-instance batch entry point: the same results,
field for field, from pageable and from pinned matrices; NaN probabilities and bad terminals
rejected; exhaustive instances handed to the whole-GPU engine with their own row."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("R", "esp", "nodes", "leaves", "dead_ends", "spilled", "queued", "iterations", "max_queue_items", "stop",
          "engine", "kernel")


@pytest.fixture(scope="module")
def ctx(engine_lib):
    c = engine_lib.Context(0)
    yield c
    c.close()


def _k15(n, seed0=0):
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(15, p_range=(0.9, 0.99), seed=seed0 + s) for s in range(n)]
    return gs[0], np.stack([g.edge_p for g in gs]), gs


def _same(a, b):
    for f in FIELDS:
        assert getattr(a, f) == getattr(b, f), (f, getattr(a, f), getattr(b, f))


@pytest.mark.parametrize("kw", [dict(target_width=1e-6, order="waves"),
                                dict(target_width=1e-6, order="maxmass", bucket_shift=1, n_buckets=64),
                                dict(target_width=1e-7, order="waves", small_kernel="group")])
def test_matrix_equals_per_instance_batch(ctx, engine_lib, kw):
    topo, pm, gs = _k15(300)
    srcs = np.zeros(len(gs), np.int32)
    dsts = np.full(len(gs), 14, np.int32)
    ref = ctx.reliability_batch(gs, srcs, dsts, **kw)
    mb = engine_lib.MatrixBatch(topo, pm, srcs, dsts)
    for _ in range(2):
        got = ctx.run_matrix(mb, **kw)
        for a, b in zip(got, ref):
            _same(a, b)


def test_matrix_pinned_and_pipelined(ctx, engine_lib):
    torch = pytest.importorskip("torch")
    topo, pm, gs = _k15(512, seed0=1000)
    pinned = torch.from_numpy(pm).pin_memory()
    mbs = [engine_lib.MatrixBatch(topo, pinned.data_ptr(), 0, 14, n=len(gs)),
           engine_lib.MatrixBatch(topo, pm, 0, 14)]
    ref = ctx.reliability_batch(gs, [0] * len(gs), [14] * len(gs), target_width=1e-6, order="waves")
    pending = None
    for k in range(6):                           # two batches in flight, alternating
        t = ctx.submit_matrix(mbs[k % 2], target_width=1e-6, order="waves")
        if pending is not None:
            ctx.wait(pending[0])
            for i in range(0, len(gs), 7):
                _same(engine_lib.Result.from_raw(pending[1].res[i]), ref[i])
        pending = (t, mbs[k % 2])
    ctx.wait(pending[0])


def test_matrix_exhaustive_hand_over(ctx, engine_lib, oracle):
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(10, p_range=(0.5, 0.95), seed=s) for s in range(3)]
    pm = np.stack([g.edge_p for g in gs])
    got = ctx.run_matrix(engine_lib.MatrixBatch(gs[0], pm, 0, 9))
    for g, r in zip(gs, got):
        o = oracle.run(g, 0, 9)
        assert r.engine == "grid" and (r.nodes, r.paths, r.iterations) == (o.nodes, o.paths, o.waves)
        assert r.R == o.R


def test_matrix_rejects_bad_input(ctx, engine_lib):
    topo, pm, gs = _k15(64)
    bad = pm.copy()
    bad[37, 5] = np.nan
    with pytest.raises(engine_lib.NrError) as e:
        ctx.run_matrix(engine_lib.MatrixBatch(topo, bad, 0, 14), target_width=1e-6, order="waves")
    assert e.value.status == -1
    dsts = np.full(64, 14, np.int32)
    dsts[9] = 15
    with pytest.raises(engine_lib.NrError) as e:
        ctx.run_matrix(engine_lib.MatrixBatch(topo, pm, 0, dsts), target_width=1e-6, order="waves")
    assert e.value.status == -1
    got = ctx.run_matrix(engine_lib.MatrixBatch(topo, pm, 0, 14), target_width=1e-6, order="waves")
    ref = ctx.reliability_batch(gs, [0] * 64, [14] * 64, target_width=1e-6, order="waves")
    for a, b in zip(got, ref):
        _same(a, b)
