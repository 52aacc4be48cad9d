"""Failure paths on the GPU, made on the host side: nothing faults, traps or hangs.

* A bounded grid-barrier wait runs out: the test option test_fault = 1 makes block 0 of the
  cooperative whole-GPU launch leave before its first barrier, so the other blocks wait for
  it until timeout_ms, set the timeout status and end; the call returns NR_ERR_TIMEOUT.
* The lane kernels' self-check ends an instance: test_fault = 2 sets their step bound to one
  step, so every instance that needs two ends with the check status; the call returns
  NR_ERR_INTERNAL.
After each, the next call on the same context returns the oracle's exact result."""
import pytest

from conftest import rel_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(engine_lib):
    c = engine_lib.Context(0)
    yield c
    c.close()


def _check_k9(ctx, oracle):
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(9, p_range=(0.5, 0.95), seed=1)
    r = ctx.reliability(g, 0, 8, capacity=1 << 20)
    o = oracle.run(g, 0, 8)
    assert (r.engine, r.paths, r.nodes, r.iterations) == ("grid", o.paths, o.nodes, o.waves)
    assert rel_close(r.R, o.R, 1e-12)


def test_grid_barrier_wait_runs_out(ctx, engine_lib, oracle):
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(9, p_range=(0.5, 0.95), seed=1)
    for _ in range(2):
        with pytest.raises(engine_lib.NrError) as e:
            ctx.reliability(g, 0, 8, capacity=1 << 20, timeout_ms=20.0, test_fault=1)
        assert e.value.status == -7                      # NR_ERR_TIMEOUT
        _check_k9(ctx, oracle)                           # the context is still good


@pytest.mark.parametrize("small_kernel", ["auto", "lane1"])
def test_lane_kernel_self_check(ctx, engine_lib, oracle, small_kernel):
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(15, p_range=(0.9, 0.99), seed=s) for s in range(64)]
    kw = dict(target_width=1e-6, bucket_shift=-1, n_buckets=64, small_kernel=small_kernel)
    with pytest.raises(engine_lib.NrError) as e:
        ctx.reliability_batch(gs, [0] * 64, [14] * 64, test_fault=2, **kw)
    assert e.value.status == -8                          # NR_ERR_INTERNAL
    res = ctx.reliability_batch(gs, [0] * 64, [14] * 64, **kw)
    assert {r.kernel for r in res} == {"lane2" if small_kernel == "auto" else "lane"}
    for g, r in list(zip(gs, res))[:8]:
        o = oracle.run(g, 0, 14, target_width=1e-6)
        assert (r.nodes, r.iterations, r.queued) == (o.nodes, o.waves, o.queued)
        assert r.R == o.R and r.esp == o.esp
    _check_k9(ctx, oracle)
