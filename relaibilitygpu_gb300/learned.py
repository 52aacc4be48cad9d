"""The learned order: training data, GPU training and use of the scorer.

The scorer (csrc/nr_mlp.cuh) is an MLP 16 -> 128 -> 128 -> 128 -> 1 that
estimates a subproblem's residual reliability r(x) = P(t reachable from s |
the subproblem's fixed edges).  In NR_ORDER_LEARNED a child is queued in the
bucket of mass(x) * r_hat(x) instead of mass(x); masses, R and ESP never
depend on the scorer, so results stay exact and the bound stays rigorous.

Training data: the warp engine records every child it queues (features,
mask, mass, instance) while solving training graphs; each child's residual
reliability is then computed by solving the child as a graph of its own
(its DOWN edges at p = 0, UP edges at p = 1): exhaustively where that is
cheap (exact labels), otherwise to an ESP width of 1e-10 (label = midpoint,
error <= 5e-11).  Training runs on the GPU (nr_mlp_train: hand-written FP32
GEMM / ReLU / Adam kernels).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import engine as E
from .graphs import Graph

N_FEAT = 16
H = 128
PKG = os.path.dirname(os.path.abspath(__file__))
DEFAULT_MODEL = os.path.join(PKG, "models", "scorer.npy")


def param_count() -> int:
    return E.lib().nr_mlp_param_count()


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def init_params(seed: int = 0) -> np.ndarray:
    p = np.zeros(param_count(), dtype=np.float32)
    E._check(E.lib().nr_mlp_init(_fp(p), int(seed)))
    return p


def unpack(p: np.ndarray):
    """Views (W1, b1, W2, b2, W3, b3, w4, b4) of a flat parameter vector."""
    o = 0
    out = []
    for shape in [(H, N_FEAT), (H,), (H, H), (H,), (H, H), (H,), (H,), (1,)]:
        k = int(np.prod(shape))
        out.append(p[o:o + k].reshape(shape))
        o += k
    return out


def gpu_grad(params: np.ndarray, X: np.ndarray, y: np.ndarray, device: int = 0):
    params = np.ascontiguousarray(params, np.float32)
    X = np.ascontiguousarray(X, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    g = np.zeros_like(params)
    loss = C.c_float()
    E._check(E.lib().nr_mlp_grad(device, _fp(params), _fp(X), _fp(y), len(y), C.byref(loss), _fp(g)))
    return float(loss.value), g


def gpu_train(params: np.ndarray, X: np.ndarray, y: np.ndarray, epochs: int = 20, batch: int = 512,
              lr: float = 1e-3, weight_decay: float = 0.0, seed: int = 0, device: int = 0):
    p = np.ascontiguousarray(params, np.float32).copy()
    X = np.ascontiguousarray(X, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    losses = np.zeros(epochs, dtype=np.float32)
    E._check(E.lib().nr_mlp_train(device, _fp(p), _fp(X), _fp(y), len(y), epochs, batch, lr, weight_decay,
                                  int(seed), _fp(losses)))
    return p, losses


def gpu_infer(params: np.ndarray, X: np.ndarray, device: int = 0) -> np.ndarray:
    params = np.ascontiguousarray(params, np.float32)
    X = np.ascontiguousarray(X, np.float32)
    y = np.zeros(len(X), dtype=np.float32)
    E._check(E.lib().nr_mlp_infer(device, _fp(params), _fp(X), len(X), _fp(y)))
    return y


# ---------------------------------------------------------------------------
# FP64 reference of the network (checks the GPU kernels)
# ---------------------------------------------------------------------------
def ref_forward(params: np.ndarray, X: np.ndarray, bf16: bool = False) -> np.ndarray:
    W1, b1, W2, b2, W3, b3, w4, b4 = [a.astype(np.float64) for a in unpack(params)]
    X = X.astype(np.float64)
    if bf16:
        W1, W2, W3, X = (round_bf16(a) for a in (W1, W2, W3, X))
    a = np.maximum(X @ W1.T + b1, 0)
    if bf16:
        a = round_bf16(a)
    a = np.maximum(a @ W2.T + b2, 0)
    if bf16:
        a = round_bf16(a)
    a = np.maximum(a @ W3.T + b3, 0)
    if bf16:
        a = round_bf16(a)
    z = a @ w4 + b4[0]
    return 1.0 / (1.0 + np.exp(-z))


def ref_grad(params: np.ndarray, X: np.ndarray, y: np.ndarray):
    """Mean binary cross-entropy and its gradient, FP64."""
    W1, b1, W2, b2, W3, b3, w4, b4 = [a.astype(np.float64) for a in unpack(params)]
    X = X.astype(np.float64)
    y = y.astype(np.float64)
    B = len(y)
    z1 = X @ W1.T + b1; a1 = np.maximum(z1, 0)
    z2 = a1 @ W2.T + b2; a2 = np.maximum(z2, 0)
    z3 = a2 @ W3.T + b3; a3 = np.maximum(z3, 0)
    z4 = a3 @ w4 + b4[0]
    p = 1 / (1 + np.exp(-z4))
    loss = np.mean(np.maximum(z4, 0) - z4 * y + np.log1p(np.exp(-np.abs(z4))))
    dz4 = (p - y) / B
    g = [None] * 8
    g[6] = a3.T @ dz4
    g[7] = np.array([dz4.sum()])
    dz3 = np.outer(dz4, w4) * (z3 > 0)
    g[4] = dz3.T @ a2; g[5] = dz3.sum(0)
    dz2 = (dz3 @ W3) * (z2 > 0)
    g[2] = dz2.T @ a1; g[3] = dz2.sum(0)
    dz1 = (dz2 @ W2) * (z1 > 0)
    g[0] = dz1.T @ X; g[1] = dz1.sum(0)
    return loss, np.concatenate([a.ravel() for a in g])


def round_bf16(a: np.ndarray) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


# ---------------------------------------------------------------------------
# training data
# ---------------------------------------------------------------------------
def collect(ctx: E.Context, graphs: Sequence[Graph], srcs, dsts, max_items: int, **opts):
    """Children queued by the warp engine while solving the batch (features, masks, masses, instance ids)."""
    b = E.Batch(graphs, srcs, dsts)
    o = E.make_options(**opts)
    feat = np.zeros((max_items, N_FEAT), dtype=np.float32)
    masks = np.zeros((max_items, 32), dtype=np.uint32)
    mass = np.zeros(max_items, dtype=np.float64)
    inst = np.zeros(max_items, dtype=np.int32)
    cnt = C.c_uint64()
    E._check(E.lib().nr_collect_children(
        ctx.h, b.n, b.arr, b.s.ctypes.data_as(C.POINTER(C.c_int32)), b.d.ctypes.data_as(C.POINTER(C.c_int32)),
        0, C.byref(o), max_items, _fp(feat), masks.ctypes.data_as(C.POINTER(C.c_uint32)),
        mass.ctypes.data_as(C.POINTER(C.c_double)), inst.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(cnt),
        b.res))
    k = int(cnt.value)
    return feat[:k], masks[:k], mass[:k], inst[:k]


def subproblem_graph(g: Graph, mask_words: np.ndarray) -> Graph:
    """The subproblem as a graph of its own: DOWN edges at p = 0, UP edges at p = 1."""
    e = np.arange(g.n_edges)
    st = (mask_words[e >> 4] >> (2 * (e & 15))) & 3
    p = g.edge_p.copy()
    p[st == 0] = 0.0
    p[st == 1] = 1.0
    return Graph(g.n_nodes, g.row_ptr, g.col_idx, g.edge_id, p, name=g.name, src=g.src, dst=g.dst)


def label(ctx: E.Context, graphs: Sequence[Graph], srcs, dsts, masks: np.ndarray, inst: np.ndarray,
          exact: bool) -> np.ndarray:
    """Residual reliability of each recorded child (exhaustive, or to ESP width 1e-10)."""
    subs = [subproblem_graph(graphs[i], masks[k]) for k, i in enumerate(inst)]
    s = [srcs[i] for i in inst]
    d = [dsts[i] for i in inst]
    out = np.zeros(len(subs))
    step = 2048
    for b0 in range(0, len(subs), step):
        kw = {} if exact else dict(target_width=1e-10, bucket_shift=0, n_buckets=64)
        res = ctx.reliability_batch(subs[b0:b0 + step], s[b0:b0 + step], d[b0:b0 + step], **kw)
        out[b0:b0 + step] = [r.R + 0.5 * r.esp for r in res]
    return out


def save(params: np.ndarray, path: str = DEFAULT_MODEL) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.save(path, np.asarray(params, np.float32))


def load(path: str = DEFAULT_MODEL) -> np.ndarray:
    p = np.load(path).astype(np.float32)
    if p.shape != (param_count(),):
        raise ValueError("scorer parameter count mismatch")
    return p


def set_model(ctx: E.Context, params: np.ndarray) -> None:
    params = np.ascontiguousarray(params, np.float32)
    E._check(E.lib().nr_context_set_model(ctx.h, _fp(params)))


def training_set(ctx: E.Context, seed: int = 0, per_family: int = 40000):
    """Features and residual-reliability labels from two graph families:
    K10 with p ~ U[0.5, 0.95] (exhaustive labels) and K12..K15 with
    p ~ U[0.9, 0.99] (labels to ESP width 1e-10)."""
    from . import graphs as G
    X, Y = [], []
    fams = [
        ([G.complete(10, p_range=(0.5, 0.95), seed=seed * 100 + s) for s in range(6)], 9,
         dict(order="maxmass", target_width=1e-4, bucket_shift=0, n_buckets=64), True),
        ([G.complete(12 + s % 4, p_range=(0.9, 0.99), seed=seed * 100 + 50 + s) for s in range(64)], None,
         dict(order="maxmass", target_width=1e-9, bucket_shift=0, n_buckets=64), False),
    ]
    for gs, dst, opts, exact in fams:
        dsts = [g.n_nodes - 1 if dst is None else dst for g in gs]
        srcs = [0] * len(gs)
        feat, masks, mass, inst = collect(ctx, gs, srcs, dsts, per_family, **opts)
        rng = np.random.default_rng(seed)
        keep = rng.permutation(len(feat))[:per_family]
        y = label(ctx, gs, srcs, dsts, masks[keep], inst[keep], exact)
        X.append(feat[keep])
        Y.append(np.clip(y, 0.0, 1.0).astype(np.float32))
    return np.concatenate(X), np.concatenate(Y)


def train_default(ctx: E.Context, seed: int = 0, epochs: int = 40, path: Optional[str] = DEFAULT_MODEL):
    X, y = training_set(ctx, seed)
    p, losses = gpu_train(init_params(seed), X, y, epochs=epochs, batch=512, lr=1e-3, seed=seed)
    if path:
        save(p, path)
    return p, losses, len(y)


if __name__ == "__main__":
    import json
    import sys
    out = sys.argv[2] if len(sys.argv) > 2 else DEFAULT_MODEL
    if len(sys.argv) > 1 and sys.argv[1] == "train":
        with E.Context(0) as ctx:
            p, losses, n = train_default(ctx, path=out)
        print(json.dumps({"samples": n, "loss_first": float(losses[0]), "loss_last": float(losses[-1]),
                          "model": out}))
