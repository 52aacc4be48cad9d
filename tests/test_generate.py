"""The generator command line writes reference-format files that both loaders (the Python
parser and the C ABI's nr_graph_load) read back to the generator's own graph."""
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _gen(*args):
    r = subprocess.run([sys.executable, "-m", "relaibilitygpu_gb300.generate", *args], cwd=ROOT,
                       capture_output=True, text=True, check=True)
    return r.stdout.strip()


def _same(a, b):
    assert a.n_nodes == b.n_nodes
    for f in ("row_ptr", "col_idx", "edge_id", "edge_p"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def test_generated_files_round_trip(tmp_path, engine_lib):
    from relaibilitygpu_gb300 import graphs
    cases = [(("grid", "--rows", "3", "--cols", "4", "--p-range", "0.8", "0.99", "--seed", "3"),
              graphs.grid(3, 4, p_range=(0.8, 0.99), seed=3), "0 11"),
             (("complete", "--n", "7", "--p", "0.9"), graphs.complete(7, p=0.9), "0 6"),
             (("gnm", "--n", "12", "--m", "20", "--p-range", "0.5", "0.95", "--seed", "4"),
              graphs.gnm(12, 20, p_range=(0.5, 0.95), seed=4), None),
             (("rgg", "--n", "40", "--m", "90", "--p-range", "0.9", "0.99", "--seed", "2"),
              graphs.rgg(40, 90, p_range=(0.9, 0.99), seed=2), None)]
    for args, g, terms in cases:
        out = str(tmp_path / f"{args[0]}.txt")
        printed = _gen(*args, "-o", out)
        assert printed == (terms or f"{g.src} {g.dst}")
        _same(graphs.load_graph(out), g)
        _same(engine_lib.load_graph_file(out), g)


def test_generated_batch(tmp_path):
    from relaibilitygpu_gb300 import graphs
    d = str(tmp_path / "batch")
    _gen("batch", "--count", "16", "--seed", "5", "-o", d)
    gs = graphs.batch_instances(16, seed=5)
    lines = open(os.path.join(d, "terminals.txt")).read().split("\n")
    for g, line in zip(gs, lines):
        name, s, t = line.split()
        _same(graphs.load_graph(os.path.join(d, name)), g)
        assert (int(s), int(t)) == (g.src, g.dst)
