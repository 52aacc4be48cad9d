"""Graphs for the reliability engine: the reference file format and seeded generators.

A graph is held the way the reference's host loader holds it
(workingPad/graph.h:12-27, built at :46-145): CSR arcs as listed in the
adjacency lists, one ``edge_id`` per arc, and one probability per edge id.
Edge ids are assigned to the (min, max) node pairs in first-seen order while
the adjacency lists are scanned node by node (graph.h:77-90); mask bit order
follows those ids, so every producer of a graph here uses the same rule.

Generators use ``numpy.random.default_rng(seed)`` (PCG64), so a seed names a
graph on every platform.  Edge probabilities are FP64.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Iterable, List, Optional, Sequence, Tuple

import numpy as np


@dataclasses.dataclass
class Graph:
    """CSR graph with per-arc edge ids and per-edge probabilities."""

    n_nodes: int
    row_ptr: np.ndarray     # int32 [n_nodes + 1]
    col_idx: np.ndarray     # int32 [n_arcs]
    edge_id: np.ndarray     # int32 [n_arcs]
    edge_p: np.ndarray      # float64 [n_edges]
    name: str = ""
    src: Optional[int] = None   # suggested terminals (generators set them)
    dst: Optional[int] = None

    @property
    def n_edges(self) -> int:
        return int(self.edge_p.shape[0])

    @property
    def n_arcs(self) -> int:
        return int(self.col_idx.shape[0])

    @property
    def mask_words(self) -> int:
        return max(1, (2 * self.n_edges + 31) // 32)

    def adjacency(self) -> List[List[Tuple[int, float]]]:
        out = []
        for u in range(self.n_nodes):
            lo, hi = int(self.row_ptr[u]), int(self.row_ptr[u + 1])
            out.append([(int(self.col_idx[j]), float(self.edge_p[self.edge_id[j]])) for j in range(lo, hi)])
        return out

    def edge_list(self) -> List[Tuple[int, int]]:
        """(u, v) with u < v for every edge id, in id order."""
        pairs: List[Optional[Tuple[int, int]]] = [None] * self.n_edges
        for u in range(self.n_nodes):
            for j in range(int(self.row_ptr[u]), int(self.row_ptr[u + 1])):
                e = int(self.edge_id[j])
                if pairs[e] is None:
                    v = int(self.col_idx[j])
                    pairs[e] = (min(u, v), max(u, v))
        return [p if p is not None else (0, 0) for p in pairs]


def from_adjacency(adj: Sequence[Sequence[Tuple[int, float]]], name: str = "", directed: bool = False) -> Graph:
    """Build a Graph from adjacency lists ``adj[u] = [(v, p), ...]`` (graph.h:77-130).

    Undirected: the two arcs of an edge share the id of the first-seen (min,max) pair.
    Directed: every arc is its own edge, ids in list order (seq/GraphRP.h:131-145)."""
    n = len(adj)
    row = np.zeros(n + 1, dtype=np.int32)
    cols: List[int] = []
    eids: List[int] = []
    probs: List[float] = []
    ids = {}
    for u in range(n):
        for v, p in adj[u]:
            key = (u, v, len(cols)) if directed else (min(u, v), max(u, v))
            if key not in ids:
                ids[key] = len(probs)
                probs.append(float(p))
            cols.append(int(v))
            eids.append(ids[key])
        row[u + 1] = len(cols)
    return Graph(n, row, np.asarray(cols, dtype=np.int32), np.asarray(eids, dtype=np.int32),
                 np.asarray(probs, dtype=np.float64), name=name)


def from_edges(n: int, edges: Iterable[Tuple[int, int]], probs: Iterable[float], name: str = "") -> Graph:
    """Undirected graph from an edge list; adjacency lists sorted by neighbour."""
    adj: List[List[Tuple[int, float]]] = [[] for _ in range(n)]
    for (u, v), p in zip(edges, probs):
        adj[u].append((v, p))
        adj[v].append((u, p))
    for lst in adj:
        lst.sort()
    return from_adjacency(adj, name=name)


# ---------------------------------------------------------------------------
# reference file format: "N E [U|D]" then N lines "deg (nbr p)*"
# (workingPad/graph.h:53-75, seq/GraphRP.h:82-148)
# ---------------------------------------------------------------------------

def parse_graph_text(text: str, name: str = "") -> Graph:
    toks = text.split()
    if len(toks) < 2:
        raise ValueError("graph header needs N and E")
    n = int(toks[0])
    pos = 2
    directed = False
    if pos < len(toks) and toks[pos][:1].isalpha():
        directed = toks[pos][:1] in "Dd"
        pos += 1
    adj: List[List[Tuple[int, float]]] = []
    for u in range(n):
        if pos >= len(toks):
            raise ValueError(f"missing degree for node {u}")
        deg = int(toks[pos]); pos += 1
        lst = []
        for _ in range(deg):
            if pos + 1 >= len(toks):
                raise ValueError(f"truncated adjacency list of node {u}")
            v = int(toks[pos]); p = float(toks[pos + 1]); pos += 2
            if not 0 <= v < n:
                raise ValueError(f"neighbour {v} of node {u} out of range")
            lst.append((v, p))
        adj.append(lst)
    return from_adjacency(adj, name=name, directed=directed)


def load_graph(path: str) -> Graph:
    with open(path, "r") as f:
        return parse_graph_text(f.read(), name=path)


def from_arcs(n: int, arcs: Iterable[Tuple[int, int]], probs: Iterable[float], name: str = "") -> Graph:
    """Directed graph: arc u -> v with its own probability (and edge id, in list order per node)."""
    adj: List[List[Tuple[int, float]]] = [[] for _ in range(n)]
    for (u, v), p in zip(arcs, probs):
        adj[u].append((v, p))
    return from_adjacency(adj, name=name, directed=True)


def format_graph(g: Graph, type_char: str = "U") -> str:
    """Reference file text; the header E counts arcs (graph.h:93).  Write a directed graph
    (every arc its own edge) with type_char 'D'."""
    lines = [f"{g.n_nodes} {g.n_arcs} {type_char}"]
    for u in range(g.n_nodes):
        lo, hi = int(g.row_ptr[u]), int(g.row_ptr[u + 1])
        parts = [str(hi - lo)]
        for j in range(lo, hi):
            parts.append(f"{int(g.col_idx[j])} {repr(float(g.edge_p[g.edge_id[j]]))}")
        lines.append(" ".join(parts))
    return "\n".join(lines) + "\n"


def save_graph(g: Graph, path: str, type_char: str = "U") -> None:
    with open(path, "w") as f:
        f.write(format_graph(g, type_char))


# ---------------------------------------------------------------------------
# seeded generators
# ---------------------------------------------------------------------------

def _probs(rng: np.random.Generator, m: int, p: Optional[float], p_range: Optional[Tuple[float, float]]):
    if p_range is not None:
        return rng.uniform(p_range[0], p_range[1], size=m)
    return np.full(m, 0.5 if p is None else float(p))


def complete(n: int, p: Optional[float] = None, p_range: Optional[Tuple[float, float]] = None,
             seed: int = 0) -> Graph:
    """K_n; edge ids (u<v) in lexicographic order, as the reference COMP*.txt files give."""
    rng = np.random.default_rng(seed)
    edges = [(u, v) for u in range(n) for v in range(u + 1, n)]
    g = from_edges(n, edges, _probs(rng, len(edges), p, p_range), name=f"K{n}")
    g.src, g.dst = 0, n - 1
    return g


def grid(rows: int, cols: int, p: Optional[float] = None, p_range: Optional[Tuple[float, float]] = None,
         seed: int = 0) -> Graph:
    """rows x cols grid, row-major node ids, terminals at opposite corners."""
    rng = np.random.default_rng(seed)
    edges = []
    for r in range(rows):
        for c in range(cols):
            u = r * cols + c
            if c + 1 < cols:
                edges.append((u, u + 1))
            if r + 1 < rows:
                edges.append((u, u + cols))
    edges.sort()
    g = from_edges(rows * cols, edges, _probs(rng, len(edges), p, p_range), name=f"grid{rows}x{cols}")
    g.src, g.dst = 0, rows * cols - 1
    return g


def _connected(n: int, edges: Sequence[Tuple[int, int]]) -> bool:
    parent = list(range(n))

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for u, v in edges:
        a, b = find(u), find(v)
        if a != b:
            parent[a] = b
    return len({find(i) for i in range(n)}) == 1


def gnm(n: int, m: int, p: Optional[float] = None, p_range: Optional[Tuple[float, float]] = None,
        seed: int = 0, max_tries: int = 10000) -> Graph:
    """Connected Erdos-Renyi G(n, m) by rejection; random distinct terminals."""
    rng = np.random.default_rng(seed)
    all_pairs = [(u, v) for u in range(n) for v in range(u + 1, n)]
    m = min(m, len(all_pairs))
    for _ in range(max_tries):
        pick = rng.choice(len(all_pairs), size=m, replace=False)
        edges = sorted(all_pairs[i] for i in pick)
        if _connected(n, edges):
            break
    else:
        raise RuntimeError("no connected G(n,m) found")
    g = from_edges(n, edges, _probs(rng, m, p, p_range), name=f"gnm{n}_{m}")
    s, t = rng.choice(n, size=2, replace=False)
    g.src, g.dst = int(s), int(t)
    return g


def random_digraph(n: int, m: int, p: Optional[float] = None, p_range: Optional[Tuple[float, float]] = None,
                   seed: int = 0, max_out: int = 10, hops: int = 5) -> Graph:
    """Directed graph ('D': every arc its own edge) with m distinct arcs u -> v, u != v, and
    out-degrees of at most max_out -- the size class of a peer-to-peer overlay such as the
    reference's directed example (6301 nodes, 20777 arcs, out-degree <= 10, p = 0.5).  src is
    node 0, dst the smallest node `hops` arcs away from it (else the farthest reachable)."""
    rng = np.random.default_rng(seed)
    out = [set() for _ in range(n)]
    arcs = 0
    while arcs < m:
        u = int(rng.integers(0, n))
        v = int(rng.integers(0, n))
        if u == v or v in out[u] or len(out[u]) >= max_out:
            continue
        out[u].add(v)
        arcs += 1
    lst = [(u, v) for u in range(n) for v in sorted(out[u])]
    g = from_arcs(n, lst, _probs(rng, len(lst), p, p_range), name=f"digraph{n}_{m}")
    dist = {0: 0}
    frontier = [0]
    while frontier:
        nxt = []
        for u in frontier:
            for v in sorted(out[u]):
                if v not in dist:
                    dist[v] = dist[u] + 1
                    nxt.append(v)
        frontier = nxt
    at = sorted(v for v, d in dist.items() if d == hops)
    g.src = 0
    g.dst = at[0] if at else max(dist, key=lambda v: (dist[v], -v))
    return g


def rgg(n: int, target_edges: int, p: Optional[float] = None, p_range: Optional[Tuple[float, float]] = None,
        seed: int = 0, max_tries: int = 1000) -> Graph:
    """Random geometric graph in the unit square with exactly ``target_edges`` edges.

    The radius is the distance of the target_edges-th closest pair; points are
    resampled until the graph is connected.  Terminals are the farthest pair.
    """
    rng = np.random.default_rng(seed)
    for _ in range(max_tries):
        pts = rng.random((n, 2))
        d = np.sqrt(((pts[:, None, :] - pts[None, :, :]) ** 2).sum(-1))
        iu, ju = np.triu_indices(n, 1)
        dist = d[iu, ju]
        order = np.argsort(dist, kind="stable")[:target_edges]
        edges = sorted((int(iu[k]), int(ju[k])) for k in order)
        if _connected(n, edges):
            break
    else:
        raise RuntimeError("no connected RGG found")
    g = from_edges(n, edges, _probs(rng, len(edges), p, p_range), name=f"rgg{n}_{target_edges}")
    far = int(np.argmax(dist))
    g.src, g.dst = int(iu[far]), int(ju[far])
    return g


def batch_instances(count: int = 4096, seed: int = 0, p_range=(0.8, 0.99)) -> List[Graph]:
    """Uneven batch: half connected G(n,m) with n~U{8..20}, m=ceil(n*d/2), d~U[3,8];
    half r x c grids with r,c~U{3..6}; p~U[p_range]; random distinct terminals."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        sub = int(rng.integers(0, 2**63 - 1))
        if i % 2 == 0:
            n = int(rng.integers(8, 21))
            d = float(rng.uniform(3.0, 8.0))
            m = min(int(math.ceil(n * d / 2.0)), n * (n - 1) // 2)
            g = gnm(n, m, p_range=p_range, seed=sub)
        else:
            r = int(rng.integers(3, 7))
            c = int(rng.integers(3, 7))
            g = grid(r, c, p_range=p_range, seed=sub)
            s, t = rng.choice(r * c, size=2, replace=False)
            g.src, g.dst = int(s), int(t)
        out.append(g)
    return out
