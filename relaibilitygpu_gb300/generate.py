"""Seeded graph generators as a command line: reference-format graph files.

    python -m relaibilitygpu_gb300.generate complete --n 15 --p-range 0.9 0.99 --seed 3 -o K15.txt
    python -m relaibilitygpu_gb300.generate grid --rows 4 --cols 4 --p 0.9 -o grid4x4.txt
    python -m relaibilitygpu_gb300.generate gnm --n 20 --m 50 --p-range 0.8 0.99 --seed 1 -o g.txt
    python -m relaibilitygpu_gb300.generate rgg --n 200 --m 600 --p-range 0.9 0.99 --seed 7 -o rgg.txt
    python -m relaibilitygpu_gb300.generate batch --count 4096 --seed 0 -o batch_dir/

The files use the reference's format ("N E U" then N lines "deg (nbr p)*", where E counts
arcs: workingPad/graph.h:53-93, seq/GraphRP.h:82-148), so the reference's own programs and
this engine's loader (nr_graph_load, the network_reliability CLI) read them.  The reference
ships only complete graphs with uniform p; these generators write the seeded grids, G(n,m),
random geometric graphs and uneven batches its benchmark configurations describe.  Each run
prints the suggested terminals ("src dst") of every file it writes; a batch also writes
terminals.txt (file name, src, dst per line).
"""
from __future__ import annotations

import argparse
import os
import sys

from . import graphs as G


def _p_kw(a) -> dict:
    return {"p_range": tuple(a.p_range)} if a.p_range else {"p": a.p}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m relaibilitygpu_gb300.generate", description=__doc__.split("\n")[0])
    sub = ap.add_subparsers(dest="kind", required=True)
    for kind in ("complete", "grid", "gnm", "rgg", "batch"):
        sp = sub.add_parser(kind)
        sp.add_argument("-o", "--out", required=True, help="output file (a directory for batch)")
        sp.add_argument("--seed", type=int, default=0)
        if kind != "batch":
            sp.add_argument("--p", type=float, default=0.5, help="one probability for every edge")
            sp.add_argument("--p-range", type=float, nargs=2, metavar=("LO", "HI"),
                            help="edge probabilities ~ U[LO, HI] instead of --p")
        if kind in ("complete", "gnm", "rgg"):
            sp.add_argument("--n", type=int, required=True)
        if kind in ("gnm", "rgg"):
            sp.add_argument("--m", type=int, required=True, help="edges (rgg: target edge count)")
        if kind == "grid":
            sp.add_argument("--rows", type=int, required=True)
            sp.add_argument("--cols", type=int, required=True)
        if kind == "batch":
            sp.add_argument("--count", type=int, default=4096)
            sp.add_argument("--p-range", type=float, nargs=2, default=(0.8, 0.99), metavar=("LO", "HI"))
    a = ap.parse_args(argv)
    if a.kind == "batch":
        os.makedirs(a.out, exist_ok=True)
        gs = G.batch_instances(a.count, seed=a.seed, p_range=tuple(a.p_range))
        width = len(str(len(gs) - 1))
        with open(os.path.join(a.out, "terminals.txt"), "w") as f:
            for i, g in enumerate(gs):
                name = f"g{i:0{width}d}.txt"
                G.save_graph(g, os.path.join(a.out, name))
                f.write(f"{name} {g.src} {g.dst}\n")
        print(f"{len(gs)} graphs in {a.out} (terminals in terminals.txt)")
        return 0
    if a.kind == "complete":
        g = G.complete(a.n, seed=a.seed, **_p_kw(a))
        s, t = 0, a.n - 1
    elif a.kind == "grid":
        g = G.grid(a.rows, a.cols, seed=a.seed, **_p_kw(a))
        s, t = 0, a.rows * a.cols - 1
    elif a.kind == "gnm":
        g = G.gnm(a.n, a.m, seed=a.seed, **_p_kw(a))
        s, t = g.src, g.dst
    else:
        g = G.rgg(a.n, a.m, seed=a.seed, **_p_kw(a))
        s, t = g.src, g.dst
    G.save_graph(g, a.out)
    print(f"{s} {t}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
