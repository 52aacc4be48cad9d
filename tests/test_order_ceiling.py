"""The ceiling of the learned order, computed on the CPU with the oracle (og_order_bound).

The learned scorer may only change which queued subproblem is popped next and the order in
which a path's UNKNOWN edges are branched; it never changes masses.  For a fixed branching
rule the oracle computes, per instance, the fewest pops ANY queue order can need to reach the
target width (a certified lower bound: the k largest width reductions of the whole
decomposition tree), next to what plain max-mass pops and the breadth-first wave count (the
fewest parallel steps any schedule can need).  The printed table is the committed result:

* queue order: plain max-mass is within a few percent of the lower bound on every family, so
  no priority -- learned, exact-residual or otherwise -- can pop 5x fewer subproblems;
* branch order changes the tree itself: branching the least reliable path edge first (p_asc)
  pops ~1.4-1.7x fewer subproblems on grids and K10 and fewer on G(n,m) and RGG N=60, while it
  leaves K15 and K25 unchanged (and, at a fixed budget, widens the RGG N=200 bracket); the
  branch order is where a learned rule has room -- but not 5x on these families."""
import numpy as np
import pytest

FAMILIES = [
    ("k15_u90_99_1e-6", lambda G, s: (G.complete(15, p_range=(0.9, 0.99), seed=s), 0, 14), 1e-6, 16),
    ("k10_u50_95_1e-4", lambda G, s: (G.complete(10, p_range=(0.5, 0.95), seed=s), 0, 9), 1e-4, 8),
    ("k25_u90_99_1e-7", lambda G, s: (G.complete(25, p_range=(0.9, 0.99), seed=s), 0, 24), 1e-7, 8),
    ("grid4x4_u80_99_1e-6", lambda G, s: (G.grid(4, 4, p_range=(0.8, 0.99), seed=s), 0, 15), 1e-6, 8),
    ("grid5x5_u80_99_1e-4", lambda G, s: (G.grid(5, 5, p_range=(0.8, 0.99), seed=s), 0, 24), 1e-4, 4),
    ("gnm20_50_u80_99_1e-6", lambda G, s: (lambda g: (g, g.src, g.dst))(G.gnm(20, 50, p_range=(0.8, 0.99), seed=s)),
     1e-6, 8),
    ("rgg60_150_u90_99_1e-4", lambda G, s: (lambda g: (g, g.src, g.dst))(G.rgg(60, 150, p_range=(0.9, 0.99), seed=s)),
     1e-4, 4),
]


@pytest.fixture(scope="module")
def table(oracle):
    from relaibilitygpu_gb300 import graphs
    rows = {}
    for name, make, target, n in FAMILIES:
        for border in ("src", "p_asc"):
            acc = {}
            for s in range(n):
                g, a, b = make(graphs, s)
                r = oracle.order_bound(g, a, b, target, branch_order=border, budget=5_000_000)
                assert r["status"] == 0, (name, s, r)
                for k, v in r.items():
                    acc[k] = acc.get(k, 0) + v
            rows[(name, border)] = {k: v / n for k, v in acc.items()}
    return rows


def test_queue_order_ceiling(table, capsys):
    with capsys.disabled():
        print("\nfamily                    branching  max-mass pops  fewest pops (any order)  ratio  "
              "breadth-first pops / waves")
        for (name, border), r in table.items():
            ratio = r["plain_pops"] / r["min_pops"]
            print(f"{name:25s} {border:9s} {r['plain_pops']:14.1f} {r['min_pops']:24.1f} {ratio:6.3f}  "
                  f"{r['bf_pops']:.1f} / {r['bf_waves']:.1f}")
    for (name, border), r in table.items():
        assert r["min_pops"] <= r["plain_pops"]
        # no queue order can pop 5x fewer subproblems than plain max-mass, for either branching
        assert r["plain_pops"] < 5 * r["min_pops"], (name, border, r)
        assert r["plain_pops"] <= 1.05 * r["min_pops"], (name, border, r)


def test_branch_order_headroom(table):
    """Branching the least reliable path edge first pops fewer subproblems on grids, where
    the queue order has no room left; still short of 5x."""
    for name in ("grid4x4_u80_99_1e-6", "grid5x5_u80_99_1e-4"):
        src, asc = table[(name, "src")], table[(name, "p_asc")]
        assert asc["plain_pops"] < 0.8 * src["plain_pops"], (name, src, asc)
        assert src["min_pops"] < 5 * asc["min_pops"]


def test_branch_orders_are_exact(oracle):
    """Every branch order is a disjoint decomposition: exhaustive R agrees with brute force."""
    from relaibilitygpu_gb300 import graphs
    rng = np.random.default_rng(5)
    for s in range(4):
        g = graphs.gnm(9, 16, p_range=(0.3, 0.95), seed=int(rng.integers(1 << 30)))
        exact = oracle.brute(g, g.src, g.dst)
        for border in ("src", "dst", "p_asc", "p_desc"):
            r = oracle.run(g, g.src, g.dst, branch_order=border)
            assert abs(r.R - exact) <= 1e-13 * exact, (border, r.R, exact)
