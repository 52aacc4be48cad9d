"""Generate the golden fixtures under tests/golden/.

Run here (where the reference tree is mounted), not on the GPU host:

    python tests/golden/make_golden.py <reference_root>   (or NR_REFERENCE_ROOT=<root>)

It writes
  graphs/*.txt   reference-format graph files produced by this repo's own
                 generators (complete graphs, the tiny hand graphs of
                 workingPad/README.md:187-204, seeded random graphs);
  golden.json    known answers:
    - "published": values printed in the reference's own run logs, with the
      log file:line they come from;
    - "analytic": closed-form values;
    - "seq_ref": outputs of the reference's seq/seq.cpp compiled from source
      by oracle/build_ref.sh and run on the seeded random graphs
      (FIFO parent rule, pre-push connectivity check);
    - "cpu_reference": outputs of workingPad/cpu_reference.cpp (float p,
      edge factoring) on the header-less tiny graphs.
Before writing, every generated graph that has a file in the reference tree
is checked to parse to the same CSR, edge ids and probabilities.
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from relaibilitygpu_gb300 import graphs as G  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NR_REFERENCE_ROOT", "")
REF_BIN = os.path.join(ROOT, "oracle", "_ref")


def hand_graphs():
    """The tiny graphs of the reference's README tables, as edge lists."""
    simple = G.from_edges(4, [(0, 1), (1, 2), (2, 3)], [0.9, 0.8, 0.7], name="test_simple")
    bridge = G.from_edges(4, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 3)], [0.9, 0.8, 0.5, 0.7, 0.6],
                          name="test_bridge")
    kite = G.from_edges(5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 3), (2, 4), (3, 4)],
                        [0.95, 0.9, 0.8, 0.85, 0.9, 0.7, 0.95], name="test_kite")
    cycle4 = G.from_edges(4, [(0, 1), (1, 2), (2, 3), (0, 3)], [0.5] * 4, name="cycle4")
    k4 = G.complete(4, p=0.5)
    k4.name = "temp4x4"
    return {"test_simple": (simple, "workingPad/test_simple.txt", "N E"),
            "test_bridge": (bridge, "workingPad/test_bridge.txt", "N E"),
            "test_kite": (kite, "workingPad/test_kite.txt", "N E"),
            "cycle4": (cycle4, "workingPad/cycle4.txt", "U"),
            "temp4x4": (k4, "workingPad/temp4x4.txt", "U")}


def complete_graphs():
    out = {}
    for name, n, p, path in [("COMP8", 8, 0.5, "workingPad/COMP8.txt"), ("COMP8-03", 8, 0.3, "workingPad/COMP8-03.txt"),
                             ("COMP9", 9, 0.5, "workingPad/COMP9.txt"), ("COMP10-05", 10, 0.5, "workingPad/COMP10-05.txt"),
                             ("COMP15-05", 15, 0.5, "workingPad/COMP15-05.txt"),
                             ("COMP25-05", 25, 0.5, "workingPad/COMP25-05.txt"),
                             ("COMP40", 40, 0.1, "workingPad/COMP40.txt")]:
        g = G.complete(n, p=p)
        g.name = name
        out[name] = (g, path, "U")
    return out


def random_graphs():
    out = {}
    for i in range(12):
        n = 6 + i % 6
        m = min(n * (n - 1) // 2, n + 4 + (i * 3) % 9)
        g = G.gnm(n, m, p_range=(0.3, 0.95), seed=1000 + i)
        out[f"gnm_{i}"] = g
    for i, (r, c) in enumerate([(3, 3), (3, 4), (4, 3), (4, 4)]):
        g = G.grid(r, c, p_range=(0.5, 0.99), seed=2000 + i)
        out[f"grid_{r}x{c}_{i}"] = g
    for i, n in enumerate([5, 6, 7, 8]):
        g = G.complete(n, p_range=(0.2, 0.9), seed=3000 + i)
        g.src, g.dst = 1, n - 2
        out[f"kn_{n}_{i}"] = g
    return out


def same_graph(a: G.Graph, b: G.Graph) -> bool:
    return (a.n_nodes == b.n_nodes and np.array_equal(a.row_ptr, b.row_ptr) and np.array_equal(a.col_idx, b.col_idx)
            and np.array_equal(a.edge_id, b.edge_id) and np.allclose(a.edge_p, b.edge_p, rtol=0, atol=1e-12))


def run_seq_ref(path: str, s: int, t: int):
    exe = os.path.join(REF_BIN, "seq_ref")
    out = subprocess.run([exe, path, str(s), str(t)], capture_output=True, text=True, timeout=600).stdout
    R = float(re.search(r"Reliability:\s+([0-9.eE+-]+)", out).group(1))
    it = int(re.search(r"Total iterations:\s+(\d+)", out).group(1))
    np_ = int(re.search(r"Paths enumerated:\s+(\d+)", out).group(1))
    return {"R": R, "iterations": it, "paths": np_}


def run_cpu_reference(path: str, s: int, t: int):
    exe = os.path.join(REF_BIN, "cpu_reference")
    out = subprocess.run([exe, path, str(s), str(t)], capture_output=True, text=True, timeout=600).stdout
    R = float(re.search(r"Reliability:\s+R = ([0-9.eE+-]+)", out).group(1))
    paths = int(re.search(r"Paths enumerated:\s+(\d+)", out).group(1))
    nodes = int(re.search(r"Nodes processed:\s+(\d+)", out).group(1))
    return {"R": R, "paths": paths, "nodes": nodes}


def main():
    if not REF:
        raise SystemExit("usage: make_golden.py <reference_root>  (or set NR_REFERENCE_ROOT)")
    gdir = os.path.join(HERE, "graphs")
    os.makedirs(gdir, exist_ok=True)
    have_ref = os.path.isdir(REF)
    if not os.path.exists(os.path.join(REF_BIN, "seq_ref")) and have_ref:
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), REF], check=True)

    files = {}
    for name, (g, refpath, hdr) in {**hand_graphs(), **complete_graphs()}.items():
        if have_ref:
            r = G.load_graph(os.path.join(REF, refpath))
            assert same_graph(g, r), f"{name} differs from {refpath}"
        fn = os.path.join(gdir, name + ".txt")
        text = G.format_graph(g, "U")
        if hdr == "N E":   # the reference's README graphs carry no type character
            first, rest = text.split("\n", 1)
            text = " ".join(first.split()[:2]) + "\n" + rest
        with open(fn, "w") as f:
            f.write(text)
        files[name] = {"file": f"graphs/{name}.txt", "reference_file": refpath}
    rnd = random_graphs()
    for name, g in rnd.items():
        fn = os.path.join(gdir, name + ".txt")
        G.save_graph(g, fn, "U")
        files[name] = {"file": f"graphs/{name}.txt", "src": g.src, "dst": g.dst}

    golden = {
        "files": files,
        "published": {
            "COMP8": {"src": 0, "dst": 7, "R": 0.98257344961166381836, "paths": 26830, "nodes": 53660,
                      "iterations": 23, "max_queue_items": 8160,
                      "source": ["original/resultsSeq.txt:7-9", "workingPad/output_noMaxMem_forkPath.txt:18-21"]},
            "COMP8-03": {"src": 0, "dst": 7, "R": 0.78581417953993681902, "paths": 26830, "nodes": 53660,
                         "iterations": 23, "max_queue_items": 8160,
                         "source": ["seq/resultsSeq_forkPath.txt:50", "workingPad/output_noMaxMem_forkPath.txt:41-44"]},
            "COMP9": {"src": 0, "dst": 8, "R": 0.99169051996432244778, "paths": 412015, "nodes": 824030,
                      "iterations": 30, "max_queue_items": 104160,
                      "source": ["seq/resultsSeq_forkPath.txt:74-80", "workingPad/output_noMaxMem_forkPath.txt:64-67"]},
            "COMP10-05": {"src": 0, "dst": 9, "R": 0.99596245255088433623, "paths": 7433032, "nodes": 14866064,
                          "iterations": 38, "max_queue_items": 1596000,
                          "source": ["seq/resultsSeq_forkPath.txt:104-110",
                                     "workingPad/output_maxMem_forkPath.txt:87-90"]},
            "COMP10-05_cap1M": {"src": 0, "dst": 9, "capacity": 1048576, "R": 0.995959559675,
                                "R_plus_esp": 0.995969373554, "source": ["workingPad/output_noMaxMem_forkPath.txt:82-91"]},
            "COMP15-05_bracket": {"src": 0, "dst": 14, "lo": 0.99984949656639954263, "hi": 0.99988836731919672474,
                                  "source": ["original/resultsSeq.txt:59-60"]},
        },
        "analytic": {
            "test_simple": {"src": 0, "dst": 3, "R": 0.504, "source": "workingPad/README.md:191-204"},
            "test_bridge": {"src": 0, "dst": 3, "R": 0.835, "source": "workingPad/README.md:191-204"},
            "cycle4": {"src": 0, "dst": 2, "R": 0.4375},
            "temp4x4": {"src": 0, "dst": 3, "R": 0.75},
        },
        "seq_ref": {},
        "cpu_reference": {},
    }
    if os.path.exists(os.path.join(REF_BIN, "seq_ref")):
        for name, g in rnd.items():
            golden["seq_ref"][name] = {"src": g.src, "dst": g.dst,
                                       **run_seq_ref(os.path.join(gdir, name + ".txt"), g.src, g.dst)}
        for name in ["COMP8", "COMP8-03", "COMP9"]:
            d = golden["published"][name]
            golden["seq_ref"][name] = {"src": d["src"], "dst": d["dst"],
                                       **run_seq_ref(os.path.join(gdir, name + ".txt"), d["src"], d["dst"])}
        for name, (s, t) in {"test_simple": (0, 3), "test_bridge": (0, 3), "test_kite": (0, 4)}.items():
            golden["cpu_reference"][name] = {"src": s, "dst": t,
                                             **run_cpu_reference(os.path.join(gdir, name + ".txt"), s, t)}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "golden.json"), len(files), "graphs")


if __name__ == "__main__":
    main()
