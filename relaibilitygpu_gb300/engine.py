"""ctypes binding of the engine's C ABI (include/nr.h).

This is the host-side mirror of the reference's `network_reliability`
driver (workingPad/main.cu:795-1072): the same arguments (graph, src, dst,
queue capacity, truncation eps) and the same result fields.  The CUDA
library is required: if libnr.so is missing or cannot load, every call
raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
from typing import Optional, Sequence

import numpy as np

from .graphs import Graph

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libnr.so")

NR_OK = 0
STATUS = {
    0: "NR_OK", -1: "NR_ERR_INVALID", -2: "NR_ERR_IO", -3: "NR_ERR_PARSE", -4: "NR_ERR_UNSUPPORTED",
    -5: "NR_ERR_CUDA", -6: "NR_ERR_NOMEM", -7: "NR_ERR_TIMEOUT", -8: "NR_ERR_INTERNAL",
}
ORDERS = {"auto": 0, "waves": 1, "maxmass": 2, "learned": 3}
BRANCHING = {"path": 0, "fork": 1}
BRANCH_ORDERS = {"src": 0, "dst": 1, "p_asc": 2, "p_desc": 3, "learned": 4}
ENGINES = {1: "grid", 2: "warp"}
KERNELS = {0: "", 1: "group", 2: "lane", 3: "lane2", 4: "block"}     # the warp engine's kernel
SMALL_KERNELS = {"auto": 0, "group": 1, "lane1": 2}


class NrError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {msg}")


class NrGraph(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int32), ("n_edges", C.c_int32), ("n_arcs", C.c_int32),
        ("row_ptr", C.POINTER(C.c_int32)), ("col_idx", C.POINTER(C.c_int32)),
        ("edge_id", C.POINTER(C.c_int32)), ("edge_p", C.POINTER(C.c_double)),
    ]


class NrOptions(C.Structure):
    _fields_ = [
        ("truncation_eps", C.c_double), ("target_width", C.c_double), ("order", C.c_int32),
        ("bucket_shift", C.c_int32), ("n_buckets", C.c_int32), ("device", C.c_int32),
        ("blocks_per_sm", C.c_int32), ("warps_per_block", C.c_int32), ("timeout_ms", C.c_double),
        ("verbose", C.c_int32), ("test_fault", C.c_int32), ("max_nodes", C.c_uint64),
        ("pages_per_warp", C.c_int32), ("branching", C.c_int32), ("small_kernel", C.c_int32),
        ("lane_slots", C.c_int32), ("branch_order", C.c_int32), ("handover_pages", C.c_int32),
    ]


class NrResult(C.Structure):
    _fields_ = [
        ("R", C.c_double), ("R_plus_esp", C.c_double), ("esp", C.c_double), ("trunc_bound", C.c_double),
        ("paths", C.c_uint64), ("nodes", C.c_uint64), ("leaves", C.c_uint64), ("dead_ends", C.c_uint64),
        ("truncated", C.c_uint64), ("spilled", C.c_uint64), ("queued", C.c_uint64),
        ("iterations", C.c_int32), ("n_nodes", C.c_int32), ("n_edges", C.c_int32),
        ("src", C.c_int32), ("dst", C.c_int32), ("mask_words", C.c_int32),
        ("max_queue_items", C.c_uint64), ("max_queue_mb", C.c_double), ("ms", C.c_double),
        ("time_to_bound_ms", C.c_double), ("engine", C.c_int32), ("grid_blocks", C.c_int32),
        ("block_threads", C.c_int32), ("item_bytes", C.c_int32), ("capacity", C.c_uint64),
        ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64), ("stop", C.c_int32), ("kernel", C.c_int32),
        ("reserved", C.c_int32 * 2),
    ]


# every symbol include/nr.h declares
EXPORTS = [
    "nr_options_default", "nr_status_string", "nr_abi_version", "nr_graph_load", "nr_graph_free",
    "nr_initial_mask", "nr_context_create", "nr_context_destroy", "nr_reliability", "nr_reliability_ctx",
    "nr_reliability_batch", "nr_batch_submit", "nr_batch_wait", "nr_format_result", "nr_reliability_noalloc", "nr_autotune",
    "nr_mlp_param_count", "nr_mlp_init", "nr_mlp_grad", "nr_mlp_train", "nr_mlp_infer", "nr_context_set_model",
    "nr_collect_children", "nr_checkpoint_save", "nr_checkpoint_resume", "nr_reliability_kterminal",
    "nr_batch_submit_matrix", "nr_reliability_batch_matrix",
]

_lib_handle: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    """Load libnr.so (raises if it is missing; there is no fallback)."""
    global _lib_handle
    if _lib_handle is not None:
        return _lib_handle
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with relaibilitygpu_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    L.nr_options_default.argtypes = [C.POINTER(NrOptions)]
    L.nr_options_default.restype = None
    L.nr_status_string.argtypes = [C.c_int]
    L.nr_status_string.restype = C.c_char_p
    L.nr_abi_version.restype = C.c_int
    L.nr_graph_load.argtypes = [C.c_char_p, C.POINTER(NrGraph)]
    L.nr_graph_load.restype = C.c_int
    L.nr_graph_free.argtypes = [C.POINTER(NrGraph)]
    L.nr_graph_free.restype = None
    L.nr_initial_mask.argtypes = [C.POINTER(NrGraph), C.POINTER(C.c_uint32), C.c_int]
    L.nr_initial_mask.restype = C.c_int
    L.nr_context_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    L.nr_context_create.restype = C.c_int
    L.nr_context_destroy.argtypes = [C.c_void_p]
    L.nr_context_destroy.restype = None
    L.nr_reliability.argtypes = [C.POINTER(NrGraph), C.c_int, C.c_int, C.c_uint64, C.POINTER(NrOptions),
                                 C.POINTER(NrResult)]
    L.nr_reliability.restype = C.c_int
    L.nr_reliability_ctx.argtypes = [C.c_void_p, C.POINTER(NrGraph), C.c_int, C.c_int, C.c_uint64,
                                     C.POINTER(NrOptions), C.POINTER(NrResult)]
    L.nr_reliability_ctx.restype = C.c_int
    L.nr_reliability_batch.argtypes = [C.c_void_p, C.c_int, C.POINTER(NrGraph), C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int32), C.c_uint64, C.POINTER(NrOptions),
                                       C.POINTER(NrResult)]
    L.nr_reliability_batch.restype = C.c_int
    L.nr_batch_submit.argtypes = [C.c_void_p, C.c_int, C.POINTER(NrGraph), C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int32), C.c_uint64, C.POINTER(NrOptions), C.POINTER(NrResult),
                                  C.c_void_p, C.POINTER(C.c_int64)]
    L.nr_batch_submit.restype = C.c_int
    L.nr_batch_wait.argtypes = [C.c_void_p, C.c_int64]
    L.nr_batch_wait.restype = C.c_int
    L.nr_batch_submit_matrix.argtypes = [C.c_void_p, C.POINTER(NrGraph), C.c_int, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_uint64, C.POINTER(NrOptions), C.POINTER(NrResult),
                                         C.c_void_p, C.POINTER(C.c_int64)]
    L.nr_batch_submit_matrix.restype = C.c_int
    L.nr_reliability_batch_matrix.argtypes = [C.c_void_p, C.POINTER(NrGraph), C.c_int, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_uint64, C.POINTER(NrOptions), C.POINTER(NrResult)]
    L.nr_reliability_batch_matrix.restype = C.c_int
    L.nr_reliability_noalloc.argtypes = [C.POINTER(NrGraph), C.c_int, C.c_int, C.POINTER(NrOptions),
                                         C.POINTER(NrResult)]
    L.nr_reliability_noalloc.restype = C.c_int
    L.nr_autotune.argtypes = [C.c_void_p, C.c_int, C.POINTER(NrGraph), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                              C.c_uint64, C.POINTER(NrOptions), C.POINTER(NrOptions), C.POINTER(C.c_double)]
    L.nr_autotune.restype = C.c_int
    fp = C.POINTER(C.c_float)
    L.nr_mlp_param_count.restype = C.c_int
    L.nr_mlp_init.argtypes = [fp, C.c_uint64]
    L.nr_mlp_init.restype = C.c_int
    L.nr_mlp_grad.argtypes = [C.c_int, fp, fp, fp, C.c_int, fp, fp]
    L.nr_mlp_grad.restype = C.c_int
    L.nr_mlp_train.argtypes = [C.c_int, fp, fp, fp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_uint64, fp]
    L.nr_mlp_train.restype = C.c_int
    L.nr_mlp_infer.argtypes = [C.c_int, fp, fp, C.c_int, fp]
    L.nr_mlp_infer.restype = C.c_int
    L.nr_context_set_model.argtypes = [C.c_void_p, fp]
    L.nr_context_set_model.restype = C.c_int
    L.nr_collect_children.argtypes = [C.c_void_p, C.c_int, C.POINTER(NrGraph), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int32), C.c_uint64, C.POINTER(NrOptions), C.c_uint64, fp,
                                      C.POINTER(C.c_uint32), C.POINTER(C.c_double), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_uint64), C.POINTER(NrResult)]
    L.nr_collect_children.restype = C.c_int
    L.nr_reliability_kterminal.argtypes = [C.c_void_p, C.POINTER(NrGraph), C.POINTER(C.c_int32), C.c_int,
                                           C.c_uint64, C.POINTER(NrOptions), C.POINTER(NrResult)]
    L.nr_reliability_kterminal.restype = C.c_int
    L.nr_checkpoint_save.argtypes = [C.c_void_p, C.c_char_p]
    L.nr_checkpoint_save.restype = C.c_int
    L.nr_checkpoint_resume.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(NrGraph), C.c_int, C.c_int, C.c_uint64,
                                       C.POINTER(NrOptions), C.POINTER(NrResult)]
    L.nr_checkpoint_resume.restype = C.c_int
    L.nr_format_result.argtypes = [C.POINTER(NrResult), C.c_char_p, C.c_size_t]
    L.nr_format_result.restype = C.c_int
    _lib_handle = L
    return L


@dataclasses.dataclass
class Result:
    R: float
    R_plus_esp: float
    esp: float
    trunc_bound: float
    paths: int
    nodes: int
    leaves: int
    dead_ends: int
    truncated: int
    spilled: int
    queued: int
    iterations: int
    n_nodes: int
    n_edges: int
    src: int
    dst: int
    mask_words: int
    max_queue_items: int
    max_queue_mb: float
    ms: float
    time_to_bound_ms: float
    engine: str
    grid_blocks: int
    block_threads: int
    item_bytes: int
    capacity: int
    h2d_bytes: int
    d2h_bytes: int
    stop: int
    kernel: str = ""
    _raw: NrResult = dataclasses.field(repr=False, default=None)

    @staticmethod
    def from_raw(r: NrResult) -> "Result":
        kw = {f: getattr(r, f) for f, _ in NrResult._fields_ if f != "reserved"}
        kw["engine"] = ENGINES.get(kw["engine"], str(kw["engine"]))
        kw["kernel"] = KERNELS.get(kw["kernel"], str(kw["kernel"]))
        return Result(_raw=r, **kw)

    def block(self) -> str:
        """The reference's result block text (workingPad/main.cu:1037-1056)."""
        buf = C.create_string_buffer(4096)
        lib().nr_format_result(C.byref(self._raw), buf, len(buf))
        return buf.value.decode()


class _GraphView:
    """Keeps the numpy arrays alive while C holds pointers into them.

    `shared` maps a topology (node count and the CSR / edge-id bytes) to the
    structural arrays of the first view that had it: views of graphs with the
    same topology then hand the engine the same pointers, and the batch entry
    point keeps one copy of the structural tables for each run of them
    without comparing the arrays."""

    def __init__(self, g: Graph, shared: Optional[dict] = None):
        self.row = np.ascontiguousarray(g.row_ptr, dtype=np.int32)
        self.col = np.ascontiguousarray(g.col_idx, dtype=np.int32)
        self.eid = np.ascontiguousarray(g.edge_id, dtype=np.int32)
        self.p = np.ascontiguousarray(g.edge_p, dtype=np.float64)
        if shared is not None:
            key = (int(g.n_nodes), self.row.tobytes(), self.col.tobytes(), self.eid.tobytes())
            first = shared.setdefault(key, (self.row, self.col, self.eid))
            self.row, self.col, self.eid = first
        self.c = NrGraph(
            int(g.n_nodes), int(self.p.shape[0]), int(self.col.shape[0]),
            self.row.ctypes.data_as(C.POINTER(C.c_int32)), self.col.ctypes.data_as(C.POINTER(C.c_int32)),
            self.eid.ctypes.data_as(C.POINTER(C.c_int32)), self.p.ctypes.data_as(C.POINTER(C.c_double)))


def make_options(eps: float = 0.0, target_width: float = 0.0, order: str = "auto", bucket_shift: int = 2,
                 n_buckets: int = 256, device: int = 0, blocks_per_sm: int = 0, warps_per_block: int = 0,
                 timeout_ms: float = 60000.0, max_nodes: int = 0, pages_per_warp: int = 0, branching: str = "path",
                 small_kernel: str = "auto", lane_slots: int = 0, test_fault: int = 0,
                 branch_order: str = "src", handover_pages: int = 0) -> NrOptions:
    o = NrOptions()
    lib().nr_options_default(C.byref(o))
    o.truncation_eps = float(eps)
    o.target_width = float(target_width)
    o.order = ORDERS[order] if isinstance(order, str) else int(order)
    o.bucket_shift = int(bucket_shift)
    o.n_buckets = int(n_buckets)
    o.device = int(device)
    o.blocks_per_sm = int(blocks_per_sm)
    o.warps_per_block = int(warps_per_block)
    o.timeout_ms = float(timeout_ms)
    o.max_nodes = int(max_nodes)
    o.pages_per_warp = int(pages_per_warp)
    o.branching = BRANCHING[branching] if isinstance(branching, str) else int(branching)
    o.small_kernel = SMALL_KERNELS[small_kernel] if isinstance(small_kernel, str) else int(small_kernel)
    o.lane_slots = int(lane_slots)
    o.test_fault = int(test_fault)
    o.branch_order = BRANCH_ORDERS[branch_order] if isinstance(branch_order, str) else int(branch_order)
    o.handover_pages = int(handover_pages)
    return o


def options_dict(o: NrOptions) -> dict:
    """Keyword arguments of make_options that reproduce an NrOptions."""
    inv = {v: k for k, v in ORDERS.items()}
    return dict(eps=o.truncation_eps, target_width=o.target_width, order=inv.get(o.order, "auto"),
                bucket_shift=o.bucket_shift, n_buckets=o.n_buckets, device=o.device,
                blocks_per_sm=o.blocks_per_sm, warps_per_block=o.warps_per_block, timeout_ms=o.timeout_ms,
                max_nodes=o.max_nodes, pages_per_warp=o.pages_per_warp,
                branching={v: k for k, v in BRANCHING.items()}.get(o.branching, "path"),
                small_kernel={v: k for k, v in SMALL_KERNELS.items()}.get(o.small_kernel, "auto"),
                lane_slots=o.lane_slots, test_fault=o.test_fault,
                branch_order={v: k for k, v in BRANCH_ORDERS.items()}.get(o.branch_order, "src"),
                handover_pages=o.handover_pages)


def _check(rc: int) -> None:
    if rc != NR_OK:
        raise NrError(rc, lib().nr_status_string(rc).decode())


class Context:
    """Reusable device state (queue buffers, stream); one call at a time."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        _check(lib().nr_context_create(int(device), C.byref(h)))
        self.h = h
        self._opt_cache: dict = {}

    def close(self) -> None:
        if self.h:
            lib().nr_context_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reliability(self, g: Graph, src: int, dst: int, capacity: int = 0, **opts) -> Result:
        gv = _GraphView(g)
        o = make_options(**opts)
        r = NrResult()
        _check(lib().nr_reliability_ctx(self.h, C.byref(gv.c), int(src), int(dst), int(capacity),
                                        C.byref(o), C.byref(r)))
        return Result.from_raw(r)

    def reliability_batch(self, graphs: Sequence[Graph], srcs, dsts, capacity: int = 0, **opts):
        return self.run_batch(Batch(graphs, srcs, dsts), capacity=capacity, **opts)

    def reliability_kterminal(self, g: Graph, terminals, capacity: int = 0, **opts) -> Result:
        """K-terminal reliability of `terminals` (all joined to terminals[0]), nr_reliability_kterminal."""
        gv = _GraphView(g)
        t = np.ascontiguousarray(terminals, dtype=np.int32)
        o = make_options(**opts)
        r = NrResult()
        _check(lib().nr_reliability_kterminal(self.h, C.byref(gv.c), t.ctypes.data_as(C.POINTER(C.c_int32)), len(t),
                                              int(capacity), C.byref(o), C.byref(r)))
        return Result.from_raw(r)

    def checkpoint_save(self, path: str) -> None:
        """Write the last bucketed whole-GPU run's queue and sums (nr_checkpoint_save)."""
        _check(lib().nr_checkpoint_save(self.h, path.encode()))

    def checkpoint_resume(self, path: str, g: Graph, src: int, dst: int, capacity: int = 0, **opts) -> Result:
        """Continue a checkpointed run (nr_checkpoint_resume) with these options."""
        gv = _GraphView(g)
        o = make_options(**opts)
        r = NrResult()
        _check(lib().nr_checkpoint_resume(self.h, path.encode(), C.byref(gv.c), int(src), int(dst), int(capacity),
                                          C.byref(o), C.byref(r)))
        return Result.from_raw(r)

    def submit(self, batch: "Batch", capacity: int = 0, after_stream: int = 0, options: Optional[NrOptions] = None,
               **opts) -> int:
        """Queue a prepared batch with nr_batch_submit and return its ticket.

        The batch's tables are built before this returns; the GPU work runs
        while the caller goes on (for example to submit the next batch).
        `after_stream` is a raw cudaStream_t (e.g. torch's
        `torch.cuda.current_stream().cuda_stream`): the upload starts after the
        work already queued there.  The batch's results are valid after
        wait(ticket); do not resubmit the same Batch object before that.  `options` (from
        make_options) replaces the keyword options: a loop of calls then builds them once."""
        o = options if options is not None else self._options(opts)
        t = C.c_int64()
        _check(lib().nr_batch_submit(self.h, batch.n, batch.arr, batch.sp, batch.dp, int(capacity), C.byref(o),
                                     batch.res, C.c_void_p(after_stream or None), C.byref(t)))
        return t.value

    def _options(self, opts: dict) -> NrOptions:
        """make_options(**opts), kept per keyword set: a stream of calls with the same options
        (the batch loop of a service) does not rebuild the struct each time."""
        key = tuple(sorted(opts.items()))
        o = self._opt_cache.get(key)
        if o is None:
            if len(self._opt_cache) > 64:
                self._opt_cache.clear()
            o = self._opt_cache[key] = make_options(**opts)
        return o

    def submit_matrix(self, mb: "MatrixBatch", capacity: int = 0, after_stream: int = 0,
                      options: Optional[NrOptions] = None, **opts) -> int:
        """Queue a MatrixBatch with nr_batch_submit_matrix and return its ticket (results in
        mb.res after wait(ticket))."""
        o = options if options is not None else self._options(opts)
        t = C.c_int64()
        _check(lib().nr_batch_submit_matrix(self.h, C.byref(mb.view.c), mb.n, C.c_void_p(mb.p_addr),
                                            C.c_void_p(mb.s.ctypes.data), C.c_void_p(mb.d.ctypes.data),
                                            int(capacity), C.byref(o), mb.res, C.c_void_p(after_stream or None),
                                            C.byref(t)))
        return t.value

    def run_matrix(self, mb: "MatrixBatch", capacity: int = 0, raw: bool = False, **opts):
        """Solve a MatrixBatch with nr_reliability_batch_matrix."""
        o = self._options(opts)
        _check(lib().nr_reliability_batch_matrix(self.h, C.byref(mb.view.c), mb.n, C.c_void_p(mb.p_addr),
                                                 C.c_void_p(mb.s.ctypes.data), C.c_void_p(mb.d.ctypes.data),
                                                 int(capacity), C.byref(o), mb.res))
        if raw:
            return mb.res
        return [Result.from_raw(mb.res[i]) for i in range(mb.n)]

    def wait(self, ticket: int) -> None:
        """Finish a submitted batch (nr_batch_wait): its Batch.res is filled."""
        _check(lib().nr_batch_wait(self.h, int(ticket)))

    def run_batch(self, batch: "Batch", capacity: int = 0, raw: bool = False, **opts):
        """Solve a prepared batch (host arrays marshalled once) with nr_reliability_batch."""
        o = self._options(opts)
        _check(lib().nr_reliability_batch(self.h, batch.n, batch.arr, batch.sp, batch.dp, int(capacity), C.byref(o),
                                          batch.res))
        if raw:
            return batch.res
        return [Result.from_raw(batch.res[i]) for i in range(batch.n)]


def autotune(ctx: "Context", batch: "Batch", capacity: int = 0, **opts):
    """Pick warp-engine settings for a batch with nr_autotune; returns (options dict, device ms)."""
    o = make_options(**opts)
    best = NrOptions()
    ms = C.c_double()
    _check(lib().nr_autotune(ctx.h, batch.n, batch.arr, batch.s.ctypes.data_as(C.POINTER(C.c_int32)),
                             batch.d.ctypes.data_as(C.POINTER(C.c_int32)), int(capacity), C.byref(o),
                             C.byref(best), C.byref(ms)))
    return options_dict(best), ms.value


class MatrixBatch:
    """One topology with a matrix of probability sets (nr_batch_submit_matrix): instance i has
    edge probabilities p[i] and terminals srcs[i], dsts[i] (scalars: the same for every one).

    `p` is a float64 array [n, n_edges] (C order), or the int address of such a matrix (e.g. a
    pinned torch tensor's data_ptr(), which makes the upload a plain DMA) with n given."""

    def __init__(self, topology: Graph, p, srcs, dsts, n: Optional[int] = None):
        self.view = _GraphView(topology)
        if isinstance(p, int):
            if n is None:
                raise ValueError("n is needed with a matrix address")
            self.p_addr, self.n, self._p = p, int(n), None
        else:
            self._p = np.ascontiguousarray(p, dtype=np.float64)
            if self._p.ndim != 2 or self._p.shape[1] != topology.n_edges:
                raise ValueError("p must be [n_instances, n_edges]")
            self.n = self._p.shape[0]
            self.p_addr = self._p.ctypes.data
        self.s = np.ascontiguousarray(np.broadcast_to(np.asarray(srcs, dtype=np.int32), (self.n,)))
        self.d = np.ascontiguousarray(np.broadcast_to(np.asarray(dsts, dtype=np.int32), (self.n,)))
        self.res = (NrResult * self.n)()


class Batch:
    """Host-side argument arrays of nr_reliability_batch, built once and reused."""

    def __init__(self, graphs: Sequence[Graph], srcs, dsts):
        shared: dict = {}
        self.views = [_GraphView(g, shared) for g in graphs]
        self.n = len(self.views)
        self.arr = (NrGraph * self.n)(*[v.c for v in self.views])
        self.s = np.ascontiguousarray(srcs, dtype=np.int32)
        self.d = np.ascontiguousarray(dsts, dtype=np.int32)
        self.sp = self.s.ctypes.data_as(C.POINTER(C.c_int32))     # converted once: each is ~5 us a call
        self.dp = self.d.ctypes.data_as(C.POINTER(C.c_int32))
        self.res = (NrResult * self.n)()


def reliability(g: Graph, src: int, dst: int, capacity: int = 0, **opts) -> Result:
    """One-shot solve through nr_reliability (creates and frees a context)."""
    gv = _GraphView(g)
    o = make_options(**opts)
    r = NrResult()
    _check(lib().nr_reliability(C.byref(gv.c), int(src), int(dst), int(capacity), C.byref(o), C.byref(r)))
    return Result.from_raw(r)


def reliability_noalloc(g: Graph, src: int, dst: int, **opts) -> Result:
    """Solve one instance through nr_reliability_noalloc: no device allocation.

    For callers that cannot call cudaMalloc (their device memory belongs to
    another allocator or pool).  The engine works inside a static 4 MiB device
    array per GPU; graphs need n_nodes <= 32, and a full queue spills into ESP.
    """
    gv = _GraphView(g)
    o = make_options(**opts)
    r = NrResult()
    _check(lib().nr_reliability_noalloc(C.byref(gv.c), int(src), int(dst), C.byref(o), C.byref(r)))
    return Result.from_raw(r)


def load_graph_file(path: str) -> Graph:
    """Parse a reference graph file through nr_graph_load."""
    cg = NrGraph()
    _check(lib().nr_graph_load(path.encode(), C.byref(cg)))
    try:
        n, na, ne = cg.n_nodes, cg.n_arcs, cg.n_edges
        row = np.ctypeslib.as_array(cg.row_ptr, shape=(n + 1,)).copy()
        col = np.ctypeslib.as_array(cg.col_idx, shape=(max(na, 1),))[:na].copy()
        eid = np.ctypeslib.as_array(cg.edge_id, shape=(max(na, 1),))[:na].copy()
        p = np.ctypeslib.as_array(cg.edge_p, shape=(max(ne, 1),))[:ne].copy()
    finally:
        lib().nr_graph_free(C.byref(cg))
    return Graph(n, row, col, eid, p, name=path)


def initial_mask(g: Graph) -> np.ndarray:
    gv = _GraphView(g)
    w = np.zeros(g.mask_words, dtype=np.uint32)
    _check(lib().nr_initial_mask(C.byref(gv.c), w.ctypes.data_as(C.POINTER(C.c_uint32)), len(w)))
    return w
