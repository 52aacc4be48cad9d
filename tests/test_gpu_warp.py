"""Warp-per-instance engine (bucketed max-mass queue, batches) against the oracle.

Truncated runs: the engine expands exactly the subproblems the oracle's wave
schedule expands (same buckets, same waves, same stop wave), so counts are
bit-exact, and R and ESP (exact fixed-point sums on both sides) are equal.
Exhaustive batches: counts and R bit-exact (order-independent)."""
import numpy as np
import pytest

from conftest import rel_close

pytestmark = pytest.mark.gpu

R_TOL = 1e-12


@pytest.fixture(scope="module")
def ctx(engine_lib):
    c = engine_lib.Context(0)
    yield c
    c.close()


def check_wave_parity(r, o):
    assert r.nodes == o.nodes
    assert r.leaves == o.leaves
    assert r.dead_ends == o.dead
    assert r.truncated == o.truncated
    assert r.iterations == o.waves
    assert r.max_queue_items == o.max_wave
    assert r.queued == o.queued
    assert r.R == o.R, (r.R, o.R)
    assert r.esp == o.esp, (r.esp, o.esp)


@pytest.mark.parametrize("target", [1e-3, 1e-6, 1e-9])
def test_k15_target_width(ctx, oracle, target):
    from relaibilitygpu_gb300 import graphs
    for seed in range(4):
        g = graphs.complete(15, p_range=(0.9, 0.99), seed=seed)
        r = ctx.reliability(g, 0, 14, target_width=target, bucket_shift=2, n_buckets=256)
        o = oracle.run(g, 0, 14, bucket_shift=2, n_buckets=256, target_width=target)
        assert o.status == 1
        check_wave_parity(r, o)
        assert r.esp <= target
        assert r.engine == "warp"


@pytest.mark.parametrize("shift,nb", [(-1, 64), (0, 64), (1, 128), (3, 512)])
def test_bucket_resolutions(ctx, oracle, shift, nb):
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(12, p_range=(0.7, 0.99), seed=5)
    r = ctx.reliability(g, 0, 11, target_width=1e-7, bucket_shift=shift, n_buckets=nb)
    o = oracle.run(g, 0, 11, bucket_shift=shift, n_buckets=nb if shift >= 0 else 1, target_width=1e-7)
    check_wave_parity(r, o)


def test_maxmass_to_empty_queue_is_exact(ctx, oracle, load_golden_graph, golden):
    """Max-mass order without a target runs to the empty queue: exhaustive result."""
    g = load_golden_graph("COMP8")
    r = ctx.reliability(g, 0, 7, order="maxmass", capacity=1 << 16)
    o = oracle.run(g, 0, 7, bucket_shift=2, n_buckets=256)
    check_wave_parity(r, o)
    assert rel_close(r.R, golden["published"]["COMP8"]["R"], R_TOL)
    assert r.paths == 26830 and r.nodes == 53660


def test_k25_target(ctx, oracle):
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(25, p_range=(0.9, 0.99), seed=1)
    r = ctx.reliability(g, 0, 24, target_width=1e-5)
    o = oracle.run(g, 0, 24, bucket_shift=2, n_buckets=256, target_width=1e-5)
    check_wave_parity(r, o)


def test_truncated_brackets_exact(ctx, oracle, load_golden_graph, golden):
    g = load_golden_graph("COMP9")
    exact = golden["published"]["COMP9"]["R"]
    for t in (1e-2, 1e-4, 1e-6):
        r = ctx.reliability(g, 0, 8, target_width=t, capacity=1 << 16)
        assert r.R <= exact + 1e-15 <= r.R + r.esp + 2e-15
        if r.spilled == 0:          # spilled mass stays in ESP: the target is only promised without spills
            assert r.esp <= t and r.stop == 1
        else:
            assert r.stop == 0


def test_warp_overflow_spills_and_brackets(ctx, load_golden_graph, golden):
    g = load_golden_graph("COMP9")
    exact = golden["published"]["COMP9"]["R"]
    r = ctx.reliability(g, 0, 8, order="maxmass", capacity=256)
    assert r.spilled > 0
    assert r.R <= exact + 1e-15 <= r.R + r.esp + 2e-15


def test_batch_exhaustive_matches_oracle(ctx, oracle):
    from relaibilitygpu_gb300 import graphs
    gs = graphs.batch_instances(48, seed=11)
    keep = []
    for g in gs:
        o = oracle.run(g, g.src, g.dst, max_nodes=200_000)
        if o.status == 0:
            keep.append((g, o))
    assert len(keep) >= 20
    res = ctx.reliability_batch([g for g, _ in keep], [g.src for g, _ in keep], [g.dst for g, _ in keep])
    for (g, o), r in zip(keep, res):
        assert r.paths == o.paths and r.nodes == o.nodes and r.leaves == o.leaves and r.dead_ends == o.dead
        assert r.R == o.R
        assert r.esp == 0.0


def test_batch_handover_to_grid_engine(ctx, oracle, load_golden_graph, golden):
    """An instance larger than the warp's budget is finished by the whole-GPU engine."""
    big = load_golden_graph("COMP10-05")
    small = load_golden_graph("COMP8")
    res = ctx.reliability_batch([small, big, small], [0, 0, 0], [7, 9, 7])
    assert res[0].engine == "warp" and res[2].engine == "warp"
    assert res[1].engine == "grid"
    assert res[1].paths == golden["published"]["COMP10-05"]["paths"]
    assert res[1].nodes == golden["published"]["COMP10-05"]["nodes"]
    for r in (res[0], res[2]):
        assert r.paths == 26830 and r.nodes == 53660


def test_batch_truncated_matches_oracle(ctx, oracle):
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(15, p_range=(0.9, 0.99), seed=100 + i) for i in range(64)]
    res = ctx.reliability_batch(gs, [0] * len(gs), [14] * len(gs), target_width=1e-6)
    for g, r in zip(gs, res):
        o = oracle.run(g, 0, 14, bucket_shift=2, n_buckets=256, target_width=1e-6)
        check_wave_parity(r, o)


def test_batch_mixed_classes(ctx, oracle):
    """Instances of several lane-group widths and mask sizes in one call."""
    from relaibilitygpu_gb300 import graphs
    rng = np.random.default_rng(3)
    gs = []
    for i in range(40):
        n = int(rng.integers(4, 33))
        m = int(min(n * (n - 1) // 2, n + rng.integers(0, 3 * n)))
        gs.append(graphs.gnm(n, m, p_range=(0.85, 0.99), seed=500 + i))
    res = ctx.reliability_batch(gs, [g.src for g in gs], [g.dst for g in gs], target_width=1e-5,
                                max_nodes=100_000)
    compared = 0
    for g, r in zip(gs, res):
        o = oracle.run(g, g.src, g.dst, bucket_shift=2, n_buckets=256, target_width=1e-5, max_nodes=20000)
        if o.status == 2 or r.spilled or r.stop == 3:
            continue      # larger than the quick-check budget or the warp's default pages
        check_wave_parity(r, o)
        compared += 1
    assert compared >= 20


def test_autotune_picks_valid_settings(ctx, oracle):
    from relaibilitygpu_gb300 import graphs
    import relaibilitygpu_gb300 as nr
    gs = [graphs.complete(15, p_range=(0.9, 0.99), seed=900 + i) for i in range(256)]
    b = nr.Batch(gs, [0] * len(gs), [14] * len(gs))
    best, ms = nr.autotune(ctx, b, target_width=1e-6)
    assert ms > 0
    assert best["bucket_shift"] in (-1, 0, 1, 2) and best["warps_per_block"] in (2, 4, 8)
    assert best["pages_per_warp"] in (64, 512, 4096)
    res = ctx.run_batch(b, **best)
    for g, r in zip(gs[:32], res[:32]):
        o = oracle.run(g, 0, 14, bucket_shift=best["bucket_shift"],
                       n_buckets=best["n_buckets"] if best["bucket_shift"] >= 0 else 1, target_width=1e-6)
        check_wave_parity(r, o)


@pytest.mark.parametrize("wpb", [1, 2, 8])
def test_warps_per_block(ctx, oracle, wpb):
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(12, p_range=(0.85, 0.99), seed=700 + i) for i in range(100)]
    res = ctx.reliability_batch(gs, [0] * 100, [11] * 100, target_width=1e-7, warps_per_block=wpb)
    assert res[0].block_threads == 32 * wpb
    for g, r in zip(gs, res):
        check_wave_parity(r, oracle.run(g, 0, 11, bucket_shift=2, n_buckets=256, target_width=1e-7))


def test_large_batch_host_pool(ctx, oracle):
    """A batch large enough for the host worker pool (table building in parallel)."""
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(9, p_range=(0.6, 0.99), seed=i) for i in range(3000)]
    res = ctx.reliability_batch(gs, [0] * len(gs), [8] * len(gs), target_width=1e-6, bucket_shift=1,
                                n_buckets=128)
    for i in range(0, 3000, 97):
        check_wave_parity(res[i], oracle.run(gs[i], 0, 8, bucket_shift=1, n_buckets=128, target_width=1e-6))


@pytest.mark.parametrize("wpb", [1, 4, 8])
def test_single_instance_any_block_size(ctx, oracle, wpb):
    """Single-instance calls with no capacity use the warp engine's own page default, for every block size."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(15, p_range=(0.9, 0.99), seed=44)
    for shift in (-1, 0):
        r = ctx.reliability(g, 0, 14, target_width=1e-6, bucket_shift=shift, n_buckets=64, warps_per_block=wpb)
        o = oracle.run(g, 0, 14, bucket_shift=shift, n_buckets=64 if shift >= 0 else 1, target_width=1e-6)
        check_wave_parity(r, o)
    r = ctx.reliability(g, 0, 14, target_width=1e-6, warps_per_block=wpb, pages_per_warp=8192)
    assert r.stop == 1


def test_batch_rejects_bad_instances(ctx, engine_lib):
    """Invalid probabilities, terminals or CSR arrays anywhere in a batch fail the whole call."""
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(9, p_range=(0.6, 0.99), seed=i) for i in range(600)]
    bad = graphs.complete(9, p_range=(0.6, 0.99), seed=7)
    bad.edge_p = bad.edge_p.copy()
    bad.edge_p[5] = float("nan")
    with pytest.raises(engine_lib.NrError) as e:
        ctx.reliability_batch(gs[:300] + [bad] + gs[300:], [0] * 601, [8] * 601, target_width=1e-6)
    assert e.value.status == -1
    with pytest.raises(engine_lib.NrError) as e:
        ctx.reliability_batch(gs, [0] * 599 + [9], [8] * 600, target_width=1e-6)
    assert e.value.status == -1
    broken = graphs.complete(9, p=0.9)
    broken.col_idx = broken.col_idx.copy()
    broken.col_idx[3] = 42
    with pytest.raises(engine_lib.NrError) as e:
        ctx.reliability_batch(gs[:10] + [broken], [0] * 11, [8] * 11)
    assert e.value.status == -1
    # the context stays usable
    r = ctx.reliability_batch(gs[:4], [0] * 4, [8] * 4, target_width=1e-6)
    assert all(x.stop == 1 for x in r)


def test_async_batches_match_sync(ctx, oracle):
    """nr_batch_submit / nr_batch_wait: four batches in flight on three slots (the fourth submit
    finishes the first), waits in any order, results identical to the synchronous call."""
    from relaibilitygpu_gb300 import graphs
    import relaibilitygpu_gb300 as nr
    sets = [[graphs.complete(12, p_range=(0.85, 0.99), seed=1000 * k + i) for i in range(700)] for k in range(4)]
    opts = dict(target_width=1e-6, bucket_shift=1, n_buckets=128)
    ref = [ctx.reliability_batch(gs, [0] * 700, [11] * 700, **opts) for gs in sets]
    batches = [nr.Batch(gs, [0] * 700, [11] * 700) for gs in sets]
    tickets = [ctx.submit(b, **opts) for b in batches]
    for t in (tickets[2], tickets[0], tickets[3], tickets[1]):
        ctx.wait(t)
    for b, rr in zip(batches, ref):
        got = [nr.Result.from_raw(b.res[i]) for i in range(b.n)]
        for a, r in zip(got, rr):
            assert (a.R, a.esp, a.nodes, a.paths, a.iterations, a.queued) == (r.R, r.esp, r.nodes, r.paths,
                                                                               r.iterations, r.queued)
    check_wave_parity(nr.Result.from_raw(batches[1].res[5]),
                      oracle.run(sets[1][5], 0, 11, bucket_shift=1, n_buckets=128, target_width=1e-6))
    with pytest.raises(nr.NrError):
        ctx.wait(tickets[0])                  # already waited for


def test_async_batch_ordering_and_drain(ctx):
    """The upload waits for the caller's stream; a synchronous call in between finishes the
    batch in flight first, and its wait still succeeds."""
    torch = pytest.importorskip("torch")
    from relaibilitygpu_gb300 import graphs
    import relaibilitygpu_gb300 as nr
    gs = [graphs.complete(10, p_range=(0.8, 0.99), seed=i) for i in range(300)]
    b = nr.Batch(gs, [0] * 300, [9] * 300)
    ref = ctx.reliability_batch(gs, [0] * 300, [9] * 300, target_width=1e-7)
    buf = torch.empty(64 << 20, dtype=torch.float32, device="cuda:0")
    buf.fill_(1.0)                               # queued on torch's stream, ahead of the upload
    t = ctx.submit(b, target_width=1e-7, after_stream=torch.cuda.current_stream().cuda_stream)
    single = ctx.reliability(gs[3], 0, 9, target_width=1e-7)
    ctx.wait(t)
    assert single.R == ref[3].R
    assert [b.res[i].R for i in range(300)] == [r.R for r in ref]
