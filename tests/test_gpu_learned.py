"""The learned scorer on the GPU: gradients, inference, training, and its use as a
queue priority (which must leave R and ESP exact and rigorous)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L(engine_lib):
    from relaibilitygpu_gb300 import learned
    return learned


def test_gradients_match_fp64_reference(L):
    rng = np.random.default_rng(5)
    p = L.init_params(7)
    X = rng.random((300, 16)).astype(np.float32)
    y = rng.random(300).astype(np.float32)
    loss, g = L.gpu_grad(p, X, y)
    rloss, rg = L.ref_grad(p, X, y)
    assert abs(loss - rloss) <= 1e-5 * max(1.0, abs(rloss))
    rel = np.abs(g - rg) / (np.abs(rg) + 1e-6 * np.abs(rg).max())
    assert np.median(rel) < 1e-4
    assert np.max(np.abs(g - rg)) <= 2e-4 * np.abs(rg).max()


def test_tensor_core_inference_matches_bf16_reference(L):
    rng = np.random.default_rng(6)
    p = L.init_params(9) * 0.6
    X = rng.random((1000, 16)).astype(np.float32)
    y = L.gpu_infer(p, X)
    ref = L.ref_forward(p, X, bf16=True)
    assert np.max(np.abs(y - ref)) < 5e-3
    assert np.max(np.abs(y - L.ref_forward(p, X))) < 5e-2


def test_training_reduces_loss(L):
    rng = np.random.default_rng(1)
    X = rng.random((4096, 16)).astype(np.float32)
    y = (1 / (1 + np.exp(-(X[:, 0] * 4 - 2 + X[:, 3])))).astype(np.float32)
    p0 = L.init_params(2)
    p, losses = L.gpu_train(p0, X, y, epochs=15, batch=256, lr=2e-3, seed=4)
    assert losses[-1] < losses[0]
    l0, _ = L.ref_grad(p0, X, y)
    l1, _ = L.ref_grad(p, X, y)
    assert l1 < l0


def test_collect_and_label_children(L, engine_lib, oracle):
    from relaibilitygpu_gb300 import graphs
    gs = [graphs.complete(8, p_range=(0.5, 0.95), seed=s) for s in range(4)]
    with engine_lib.Context(0) as ctx:
        feat, masks, mass, inst = L.collect(ctx, gs, [0] * 4, [7] * 4, 4000, order="maxmass")
        assert len(feat) > 100 and np.all((inst >= 0) & (inst < 4))
        assert np.all(feat[:, 15] == 1.0) and np.all((feat[:, 1] >= 0) & (feat[:, 1] <= 1))
        lab = L.label(ctx, gs, [0] * 4, [7] * 4, masks[:200], inst[:200], exact=True)
    for k in range(0, 200, 17):
        sub = L.subproblem_graph(gs[inst[k]], masks[k])
        assert lab[k] == oracle.run(sub, 0, 7).R


def test_learned_order_is_exact_and_rigorous(L, engine_lib, oracle, golden, load_golden_graph):
    """Any scorer only changes the order: exhaustive results equal the plain ones, and truncated
    results keep R <= exact <= R + ESP with ESP <= target."""
    p = L.init_params(11)
    with engine_lib.Context(0) as ctx:
        L.set_model(ctx, p)
        g = load_golden_graph("COMP8")
        r = ctx.reliability(g, 0, 7, order="learned", capacity=1 << 16)
        assert r.paths == 26830 and r.nodes == 53660 and r.R == oracle.run(g, 0, 7).R
        g9 = load_golden_graph("COMP9")
        exact = golden["published"]["COMP9"]["R"]
        for t in (1e-3, 1e-5):
            r = ctx.reliability(g9, 0, 8, order="learned", target_width=t, capacity=1 << 18)
            assert r.stop == 1 and r.esp <= t
            assert r.R <= exact + 1e-15 <= r.R + r.esp + 2e-15


def test_learned_order_needs_a_model(engine_lib):
    from relaibilitygpu_gb300 import graphs
    with engine_lib.Context(0) as ctx:
        with pytest.raises(engine_lib.NrError):
            ctx.reliability(graphs.complete(6, p=0.5), 0, 5, order="learned")


@pytest.mark.parametrize("family", ["k15_u90_99_1e-6", "k10_u50_95_1e-4"])
def test_trained_scorer_gain_over_plain_order(L, engine_lib, family, capsys):
    """What the shipped scorer gains over the plain max-mass order, on held-out seeds of the two
    training families: subproblems popped until ESP + queued <= target, summed over 128
    instances, at one bucket per factor of two (the resolution where a priority can reorder).

    Measured on a GB300: K15 p~U[0.9,0.99] to 1e-6, 3,795 subproblems either way (ratio 1.000);
    K10 p~U[0.5,0.95] to 1e-4, 139,252 plain against 178,874 learned (ratio 1.285, a loss).  On
    these families max-mass is already about the best one-step order (an exact-residual key,
    computed by brute force on the CPU, does not beat it either), so the scorer gains nothing and
    its inference makes each pop slower.  The test pins the exactness and rigour of both runs and
    bounds the loss (at most 1.5x the subproblems); the printed line is the measurement."""
    import os
    if not os.path.exists(L.DEFAULT_MODEL):
        pytest.skip("no trained scorer")
    from relaibilitygpu_gb300 import graphs
    if family.startswith("k15"):
        gs = [graphs.complete(15, p_range=(0.9, 0.99), seed=50_000 + s) for s in range(128)]
        target = 1e-6
    else:
        gs = [graphs.complete(10, p_range=(0.5, 0.95), seed=60_000 + s) for s in range(128)]
        target = 1e-4
    srcs, dsts = [0] * len(gs), [g.n_nodes - 1 for g in gs]
    opts = dict(target_width=target, bucket_shift=0, n_buckets=64, capacity=1 << 16)
    with engine_lib.Context(0) as ctx:
        plain = ctx.reliability_batch(gs, srcs, dsts, order="maxmass", **opts)
        L.set_model(ctx, L.load())
        learned = ctx.reliability_batch(gs, srcs, dsts, order="learned", **opts)
    for a, b in zip(plain, learned):
        assert a.stop == 1 and b.stop == 1 and a.esp <= target and b.esp <= target
        # both bracket the same exact value: the intervals overlap
        assert max(a.R, b.R) <= min(a.R + a.esp, b.R + b.esp) + 1e-15
    n_plain = sum(r.nodes for r in plain)
    n_learned = sum(r.nodes for r in learned)
    with capsys.disabled():
        print(f"\n[{family}] subproblems to the bound over {len(gs)} instances: plain {n_plain}, "
              f"learned {n_learned} (ratio {n_learned / n_plain:.3f})")
    assert n_learned <= 1.5 * n_plain


def test_learned_branch_order_is_exact_and_rigorous(L, engine_lib, oracle):
    """The learned branch order (NR_BORDER_LEARNED: the scorer ranks a path's UNKNOWN edges) changes
    the decomposition, never its exactness: truncated runs stop at the target and bracket the
    brute-force value, with any parameters."""
    import os
    from relaibilitygpu_gb300 import graphs
    with engine_lib.Context(0) as ctx:
        for params in ([L.load()] if os.path.exists(L.DEFAULT_MODEL) else []) + [L.init_params(3)]:
            L.set_model(ctx, params)
            for g, s, t in [(graphs.grid(4, 4, p_range=(0.6, 0.95), seed=1), 0, 15),
                            (graphs.complete(7, p_range=(0.5, 0.95), seed=2), 0, 6)]:
                exact = oracle.brute(g, s, t)
                for tw in (1e-3, 1e-6):
                    for order in ("maxmass", "learned"):
                        r = ctx.reliability(g, s, t, target_width=tw, order=order, bucket_shift=0, n_buckets=64,
                                            branch_order="learned", capacity=1 << 16)
                        assert r.stop == 1 and r.esp <= tw and r.spilled == 0
                        assert r.R <= exact * (1 + 1e-12) and exact <= (r.R + r.esp) * (1 + 1e-12)


@pytest.mark.parametrize("family", ["grid4x4_u80_99_1e-6", "k10_u50_95_1e-4", "k15_u90_99_1e-6"])
def test_branch_order_measured(L, engine_lib, family, capsys):
    """Subproblems to the bound with the plain max-mass queue under each branch order, summed over
    64 held-out instances: the reference's src-side-first order, least reliable first (p_asc), and
    the learned order.  The printed line is the measurement; the test pins rigour."""
    import os
    if not os.path.exists(L.DEFAULT_MODEL):
        pytest.skip("no trained scorer")
    from relaibilitygpu_gb300 import graphs
    if family.startswith("grid"):
        gs, target = [graphs.grid(4, 4, p_range=(0.8, 0.99), seed=70_000 + s) for s in range(64)], 1e-6
    elif family.startswith("k10"):
        gs, target = [graphs.complete(10, p_range=(0.5, 0.95), seed=60_000 + s) for s in range(64)], 1e-4
    else:
        gs, target = [graphs.complete(15, p_range=(0.9, 0.99), seed=50_000 + s) for s in range(64)], 1e-6
    srcs, dsts = [0] * len(gs), [g.n_nodes - 1 for g in gs]
    opts = dict(target_width=target, order="maxmass", bucket_shift=0, n_buckets=64, capacity=1 << 16,
                small_kernel="group")
    counts = {}
    with engine_lib.Context(0) as ctx:
        L.set_model(ctx, L.load())
        runs = {b: ctx.reliability_batch(gs, srcs, dsts, branch_order=b, **opts) for b in ("src", "p_asc", "learned")}
    for b, res in runs.items():
        for r, a in zip(res, runs["src"]):
            assert r.stop == 1 and r.esp <= target
            assert max(a.R, r.R) <= min(a.R + a.esp, r.R + r.esp) + 1e-15
        counts[b] = sum(r.nodes for r in res)
    with capsys.disabled():
        print(f"\n[{family}] subproblems to the bound over {len(gs)} instances, max-mass queue: "
              + ", ".join(f"{b} {n}" for b, n in counts.items())
              + f" (learned / src {counts['learned'] / counts['src']:.3f})")


def test_learned_branch_order_on_large_graphs(L, engine_lib):
    """Graphs above 32 nodes take the learned branch order in the bucketed whole-GPU queue: each
    run stops at its target or budget, and its bracket contains the value a tight plain run
    brackets, with the trained and with random parameters; a batch of them gives the same
    results; breadth-first waves refuse it (NR_ERR_UNSUPPORTED)."""
    import os
    from relaibilitygpu_gb300 import graphs
    cases = [graphs.rgg(40, 80, p_range=(0.85, 0.99), seed=11), graphs.rgg(60, 150, p_range=(0.9, 0.99), seed=12),
             graphs.grid(6, 6, p_range=(0.8, 0.99), seed=13), graphs.complete(40, p_range=(0.9, 0.99), seed=14)]
    ends = [(g.src, g.dst) if g.n_nodes != 40 or g.n_edges == 80 else (0, 39) for g in cases]
    kw = dict(order="maxmass", bucket_shift=2, n_buckets=255, capacity=1 << 22)
    with engine_lib.Context(0) as ctx:
        tight = [ctx.reliability(g, s, t, target_width=1e-9, max_nodes=3_000_000, **kw) for g, (s, t) in zip(cases, ends)]
        for params in ([L.load()] if os.path.exists(L.DEFAULT_MODEL) else []) + [L.init_params(4)]:
            L.set_model(ctx, params)
            one = []
            for g, (s, t), ref in zip(cases, ends, tight):
                r = ctx.reliability(g, s, t, target_width=1e-5, max_nodes=500_000, branch_order="learned", **kw)
                assert r.engine == "grid" and r.stop in (1, 3) and (r.esp <= 1e-5 or r.stop == 3)
                assert max(r.R, ref.R) <= min(r.R + r.esp, ref.R + ref.esp) + 1e-15
                one.append(r)
            res = ctx.reliability_batch(cases, [s for s, _ in ends], [t for _, t in ends], target_width=1e-5,
                                        max_nodes=500_000, branch_order="learned", **kw)
            for a, b in zip(res, one):
                assert (a.R, a.esp, a.nodes, a.iterations, a.queued) == (b.R, b.esp, b.nodes, b.iterations, b.queued)
        with pytest.raises(engine_lib.NrError):
            ctx.reliability(cases[0], ends[0][0], ends[0][1], target_width=1e-5, order="waves", branch_order="learned")
