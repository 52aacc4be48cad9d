"""CPU checks of the FP64 reference network used to check the GPU kernels."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def L(engine_lib):
    from relaibilitygpu_gb300 import learned
    return learned


def test_param_count_and_init(L):
    p = L.init_params(3)
    assert p.shape == (L.param_count(),) == (16 * 128 + 128 + 2 * (128 * 128 + 128) + 128 + 1,)
    q = L.init_params(3)
    assert np.array_equal(p, q)
    W1 = L.unpack(p)[0]
    assert abs(W1).max() <= np.sqrt(6 / 16) + 1e-6 and abs(W1).max() > 0.1


def test_reference_gradient_by_finite_differences(L):
    rng = np.random.default_rng(0)
    p = L.init_params(1).astype(np.float64) * 0.5
    X = rng.random((12, 16))
    y = rng.random(12)
    loss, g = L.ref_grad(p, X, y)
    for idx in rng.choice(len(p), 25, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[idx] += h
        pm[idx] -= h
        num = (L.ref_grad(pp, X, y)[0] - L.ref_grad(pm, X, y)[0]) / (2 * h)
        assert abs(num - g[idx]) <= 1e-6 + 1e-4 * abs(num)


def test_bf16_rounding(L):
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0], dtype=np.float32)
    r = L.round_bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12 and r[4] == 0.0


def test_subproblem_graph_fixes_edges(L, oracle):
    """A child's residual reliability = R of the graph with its DOWN edges at p=0 and UP edges at p=1."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(6, p_range=(0.3, 0.9), seed=2)
    W = g.mask_words
    m = np.zeros(W, dtype=np.uint32)
    states = [3] * g.n_edges
    states[0], states[4], states[7] = 0, 1, 0
    for e, st in enumerate(states):
        m[e >> 4] |= np.uint32(st << (2 * (e & 15)))
    sub = L.subproblem_graph(g, m)
    assert sub.edge_p[0] == 0.0 and sub.edge_p[4] == 1.0 and sub.edge_p[7] == 0.0
    assert sub.edge_p[1] == g.edge_p[1]
    # brute force over the free edges agrees with conditioning the original graph
    r = oracle.run(sub, 0, 5).R
    assert abs(r - oracle.brute(sub, 0, 5)) < 1e-14
