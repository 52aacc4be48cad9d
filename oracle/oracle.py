"""ctypes wrapper of the CPU oracle (oracle/pathdecomp.c).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker and the timed CPU port of the
reference algorithm.  The engine never imports it.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
CLI = os.path.join(HERE, "og_cli")

RULES = {"level": 0, "fifo": 1}
ORDERS = {"waves": 0, "heap": 1, "dfs": 2}


class OgGraph(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("n_edges", C.c_int32), ("n_arcs", C.c_int32),
                ("row_ptr", C.POINTER(C.c_int32)), ("col_idx", C.POINTER(C.c_int32)),
                ("edge_id", C.POINTER(C.c_int32)), ("edge_p", C.POINTER(C.c_double))]


BRANCHING = {"path": 0, "fork": 1}


class OgOpts(C.Structure):
    _fields_ = [("bfs_rule", C.c_int32), ("precheck", C.c_int32), ("order", C.c_int32),
                ("bucket_shift", C.c_int32), ("n_buckets", C.c_int32), ("threads", C.c_int32),
                ("eps", C.c_double), ("target_width", C.c_double), ("capacity", C.c_uint64),
                ("max_nodes", C.c_uint64), ("branching", C.c_int32), ("n_terminals", C.c_int32),
                ("terminals", C.c_void_p), ("branch_order", C.c_int32)]


BRANCH_ORDERS = {"src": 0, "dst": 1, "p_asc": 2, "p_desc": 3}


class OgBound(C.Structure):
    _fields_ = [("plain_pops", C.c_uint64), ("min_pops", C.c_uint64), ("bf_pops", C.c_uint64),
                ("bf_waves", C.c_uint64), ("explored", C.c_uint64), ("status", C.c_int32), ("pad", C.c_int32)]


class OgResult(C.Structure):
    _fields_ = [("R", C.c_double), ("esp", C.c_double), ("esp_spilled", C.c_double),
                ("esp_truncated", C.c_double), ("queued_mass", C.c_double),
                ("paths", C.c_uint64), ("nodes", C.c_uint64), ("leaves", C.c_uint64), ("dead", C.c_uint64),
                ("truncated", C.c_uint64), ("spilled", C.c_uint64), ("pruned", C.c_uint64),
                ("pushes", C.c_uint64), ("waves", C.c_uint64), ("max_wave", C.c_uint64),
                ("max_queued", C.c_uint64), ("queued", C.c_uint64), ("status", C.c_int32),
                ("seconds", C.c_double)]


def build() -> None:
    """Compile liboracle.so and og_cli with the oracle's Makefile."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.og_run.argtypes = [C.POINTER(OgGraph), C.c_int, C.c_int, C.POINTER(OgOpts), C.POINTER(OgResult)]
        L.og_run.restype = C.c_int
        L.og_brute.argtypes = [C.POINTER(OgGraph), C.c_int, C.c_int]
        L.og_brute.restype = C.c_double
        L.og_brute_k.argtypes = [C.POINTER(OgGraph), C.POINTER(C.c_int32), C.c_int]
        L.og_brute_k.restype = C.c_double
        L.og_bucket.argtypes = [C.c_double, C.c_int, C.c_int]
        L.og_bucket.restype = C.c_int
        L.og_run_batch.argtypes = [C.c_int, C.POINTER(OgGraph), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                   C.POINTER(OgOpts), C.POINTER(OgResult), C.c_int]
        L.og_run_batch.restype = C.c_int
        L.og_order_bound.argtypes = [C.POINTER(OgGraph), C.c_int, C.c_int, C.POINTER(OgOpts), C.c_uint64,
                                     C.POINTER(OgBound)]
        L.og_order_bound.restype = C.c_int
        L.og_default_opts.argtypes = [C.POINTER(OgOpts)]
        L.og_default_opts.restype = None
        _lib = L
    return _lib


@dataclasses.dataclass
class OracleResult:
    R: float
    esp: float
    esp_spilled: float
    esp_truncated: float
    queued_mass: float
    paths: int
    nodes: int
    leaves: int
    dead: int
    truncated: int
    spilled: int
    pruned: int
    pushes: int
    waves: int
    max_wave: int
    max_queued: int
    queued: int
    status: int
    seconds: float


class _View:
    def __init__(self, g):
        self.row = np.ascontiguousarray(g.row_ptr, dtype=np.int32)
        self.col = np.ascontiguousarray(g.col_idx, dtype=np.int32)
        self.eid = np.ascontiguousarray(g.edge_id, dtype=np.int32)
        self.p = np.ascontiguousarray(g.edge_p, dtype=np.float64)
        self.c = OgGraph(int(g.n_nodes), int(self.p.shape[0]), int(self.col.shape[0]),
                         self.row.ctypes.data_as(C.POINTER(C.c_int32)),
                         self.col.ctypes.data_as(C.POINTER(C.c_int32)),
                         self.eid.ctypes.data_as(C.POINTER(C.c_int32)),
                         self.p.ctypes.data_as(C.POINTER(C.c_double)))


def _opts(rule="level", precheck=False, order="waves", bucket_shift=-1, n_buckets=1, threads=1, eps=0.0,
          target_width=0.0, capacity=0, max_nodes=0, branching="path") -> OgOpts:
    o = OgOpts()
    lib().og_default_opts(C.byref(o))
    o.bfs_rule = RULES[rule]
    o.precheck = int(bool(precheck))
    o.order = ORDERS[order]
    o.bucket_shift = int(bucket_shift)
    o.n_buckets = int(n_buckets)
    o.threads = int(threads)
    o.eps = float(eps)
    o.target_width = float(target_width)
    o.capacity = int(capacity)
    o.max_nodes = int(max_nodes)
    o.branching = BRANCHING[branching]
    return o


class BatchArgs:
    """Host arrays for og_run_batch, built once (keeps the numpy views alive)."""

    def __init__(self, graphs, srcs, dsts):
        self.views = [_View(g) for g in graphs]
        self.n = len(self.views)
        self.arr = (OgGraph * self.n)(*[v.c for v in self.views])
        self.s = np.ascontiguousarray(srcs, dtype=np.int32)
        self.d = np.ascontiguousarray(dsts, dtype=np.int32)
        self.res = (OgResult * self.n)()


def run_batch(batch: BatchArgs, threads: int = 1, **kw):
    """Solve every instance (one worker thread per instance at a time); returns raw results."""
    o = _opts(**kw)
    rc = lib().og_run_batch(batch.n, batch.arr, batch.s.ctypes.data_as(C.POINTER(C.c_int32)),
                            batch.d.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(o), batch.res, int(threads))
    if rc != 0:
        raise ValueError("oracle rejected the batch")
    return batch.res


def run(g, src: int, dst: int, rule: str = "level", precheck: bool = False, order: str = "waves",
        bucket_shift: int = -1, n_buckets: int = 1, threads: int = 1, eps: float = 0.0,
        target_width: float = 0.0, capacity: int = 0, max_nodes: int = 0, branching: str = "path",
        terminals=None, branch_order: str = "src") -> OracleResult:
    """terminals: K-terminal reliability of this node list (src and dst are then ignored;
    terminals[0] is the search root)."""
    v = _View(g)
    o = OgOpts()
    lib().og_default_opts(C.byref(o))
    o.bfs_rule = RULES[rule]
    o.precheck = int(bool(precheck))
    o.order = ORDERS[order]
    o.bucket_shift = int(bucket_shift)
    o.n_buckets = int(n_buckets)
    o.threads = int(threads)
    o.eps = float(eps)
    o.target_width = float(target_width)
    o.capacity = int(capacity)
    o.max_nodes = int(max_nodes)
    o.branching = BRANCHING[branching]
    o.branch_order = BRANCH_ORDERS[branch_order]
    term = None
    if terminals is not None:
        term = np.ascontiguousarray(terminals, dtype=np.int32)
        o.n_terminals = len(term)
        o.terminals = term.ctypes.data
    r = OgResult()
    rc = lib().og_run(C.byref(v.c), int(src), int(dst), C.byref(o), C.byref(r))
    if rc != 0:
        raise ValueError(f"oracle rejected the instance ({rc})")
    return OracleResult(**{f: getattr(r, f) for f, _ in OgResult._fields_})


def order_bound(g, src: int, dst: int, target_width: float, branch_order: str = "src",
                budget: int = 50_000_000) -> dict:
    """The ceiling of queue orders for one branching rule (og_order_bound in oracle.h): max-mass
    pops, the fewest pops any order can need, breadth-first pops and waves (the fewest parallel
    steps any schedule can need)."""
    v = _View(g)
    o = OgOpts()
    lib().og_default_opts(C.byref(o))
    o.target_width = float(target_width)
    o.branch_order = BRANCH_ORDERS[branch_order]
    b = OgBound()
    if lib().og_order_bound(C.byref(v.c), int(src), int(dst), C.byref(o), int(budget), C.byref(b)) != 0:
        raise ValueError("oracle rejected the instance")
    return {f: int(getattr(b, f)) for f, _ in OgBound._fields_ if f != "pad"}


def brute_k(g, terminals) -> float:
    v = _View(g)
    t = np.ascontiguousarray(terminals, dtype=np.int32)
    r = lib().og_brute_k(C.byref(v.c), t.ctypes.data_as(C.POINTER(C.c_int32)), len(t))
    if r < 0:
        raise ValueError("brute force limits: n_nodes <= 64 and at most 30 uncertain edges")
    return r


def brute(g, src: int, dst: int) -> float:
    v = _View(g)
    r = lib().og_brute(C.byref(v.c), int(src), int(dst))
    if r < 0:
        raise ValueError("brute force limits: n_nodes <= 64 and at most 30 uncertain edges")
    return r


def bucket(mass: float, shift: int, n_buckets: int) -> int:
    return lib().og_bucket(float(mass), int(shift), int(n_buckets))
