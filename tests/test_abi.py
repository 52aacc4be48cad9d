"""C ABI checks that need no GPU: the library loads, exports every symbol that
include/nr.h declares, parses graph files like the reference loader, and
rejects bad input with status codes instead of exiting."""
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN_DIR, ROOT


def header_symbols():
    text = open(os.path.join(ROOT, "include", "nr.h")).read()
    return sorted(set(re.findall(r"\b(nr_[a-z_]+)\s*\(", text)))


def test_exports_every_declared_symbol(engine_lib):
    import ctypes
    L = ctypes.CDLL(engine_lib.LIB_PATH)
    syms = header_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(engine_lib.EXPORTS)
    assert engine_lib.lib().nr_abi_version() == 2


@pytest.mark.parametrize("name", ["COMP8", "COMP9", "test_simple", "test_kite", "cycle4", "gnm_3", "grid_4x4_3"])
def test_loader_matches_python_parser(engine_lib, name):
    from relaibilitygpu_gb300 import graphs
    path = os.path.join(GOLDEN_DIR, "graphs", name + ".txt")
    a = engine_lib.load_graph_file(path)
    b = graphs.load_graph(path)
    assert a.n_nodes == b.n_nodes
    for f in ("row_ptr", "col_idx", "edge_id"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert np.array_equal(a.edge_p, b.edge_p)


def test_loader_errors(engine_lib, tmp_path):
    with pytest.raises(engine_lib.NrError) as e:
        engine_lib.load_graph_file(str(tmp_path / "missing.txt"))
    assert e.value.status == -2
    bad = tmp_path / "bad.txt"
    bad.write_text("3 4 U\n2 1 0.5 9 0.5\n1 0 0.5\n0\n")
    with pytest.raises(engine_lib.NrError) as e:
        engine_lib.load_graph_file(str(bad))
    assert e.value.status == -3
    trunc = tmp_path / "trunc.txt"
    trunc.write_text("3 4 U\n2 1 0.5\n")
    with pytest.raises(engine_lib.NrError) as e:
        engine_lib.load_graph_file(str(trunc))
    assert e.value.status == -3


def test_initial_mask(engine_lib):
    from relaibilitygpu_gb300 import graphs
    g = graphs.from_edges(3, [(0, 1), (1, 2), (0, 2)], [0.0, 1.0, 0.5])
    w = engine_lib.initial_mask(g)
    # ids by adjacency scan: (0,1)=0 down, (0,2)=1 unknown, (1,2)=2 up
    assert w.tolist() == [0b011100]


def test_invalid_arguments_rejected_without_gpu(engine_lib):
    from relaibilitygpu_gb300 import graphs
    g = graphs.complete(5, p=0.5)
    for s, t in [(-1, 2), (0, 5), (7, 1)]:
        with pytest.raises(engine_lib.NrError) as e:
            engine_lib.reliability(g, s, t)
        assert e.value.status == -1
    bad = graphs.complete(4, p=0.5)
    bad.col_idx = bad.col_idx.copy()
    bad.col_idx[0] = 99
    with pytest.raises(engine_lib.NrError) as e:
        engine_lib.reliability(bad, 0, 3)
    assert e.value.status == -1


def test_no_device_is_an_error_not_a_crash(engine_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from relaibilitygpu_gb300 import graphs
    with pytest.raises(engine_lib.NrError) as e:
        engine_lib.reliability(graphs.complete(5, p=0.5), 0, 4)
    assert e.value.status in (-5, -1)


def test_format_result_layout(engine_lib):
    r = engine_lib.NrResult()
    r.R, r.R_plus_esp, r.esp, r.trunc_bound = 0.5, 0.5, 0.0, 0.0
    r.paths, r.nodes, r.iterations, r.n_nodes, r.n_edges, r.src, r.dst = 3, 7, 2, 4, 4, 0, 2
    res = engine_lib.Result.from_raw(r)
    text = res.block()
    lines = text.split("\n")
    assert lines[2] == "  Two-Terminal Network Reliability Results"
    assert "Reliability:      R(G) = 0.500000000000" in text
    assert "Paths enumerated: 3" in text and "Nodes processed:  7" in text and "Kernel iterations:2" in text


def test_status_strings(engine_lib):
    L = engine_lib.lib()
    for code in range(0, -9, -1):
        assert L.nr_status_string(code)


def test_batch_validation_on_host_pool(engine_lib):
    """Large batches validate on the context's worker threads; a bad instance is reported."""
    import torch
    from relaibilitygpu_gb300 import graphs
    if torch.cuda.is_available():
        pytest.skip("checks the no-GPU path")
    try:
        ctx = engine_lib.Context(0)
    except engine_lib.NrError as e:
        assert e.status in (-5, -1)      # no device here: context creation reports it
        return
    gs = [graphs.complete(6, p=0.5) for _ in range(2000)]
    with pytest.raises(engine_lib.NrError):
        ctx.reliability_batch(gs, [0] * 2000, [9] * 2000)


def test_cli_usage_and_errors_without_gpu(tmp_path):
    """The program's argument and file errors need no GPU: usage on too few arguments, a message
    and a non-zero exit on a missing or malformed file."""
    import subprocess
    import os
    cli = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "relaibilitygpu_gb300",
                       "network_reliability")
    if not os.path.exists(cli):
        pytest.skip("CLI not built")
    r = subprocess.run([cli], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Usage" in r.stderr and "--fork" in r.stderr
    r = subprocess.run([cli, str(tmp_path / "missing.txt"), "0", "1"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Cannot load" in r.stderr
    bad = tmp_path / "bad.txt"
    bad.write_text("3 4 U\n1 1\n")
    r = subprocess.run([cli, str(bad), "0", "1"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Cannot load" in r.stderr


def test_loader_directed_graphs(engine_lib, tmp_path):
    """nr_graph_load on a 'D' file: one edge per arc, ids in file order, as the Python parser."""
    from relaibilitygpu_gb300 import graphs
    g = graphs.from_arcs(4, [(0, 1), (1, 0), (1, 2), (2, 3), (3, 1)], [0.9, 0.8, 0.7, 0.6, 0.5])
    path = tmp_path / "d.txt"
    path.write_text(graphs.format_graph(g, "D"))
    c = engine_lib.load_graph_file(str(path))
    assert (c.n_edges, c.n_arcs) == (5, 5)
    assert np.array_equal(c.edge_id, g.edge_id) and np.array_equal(c.edge_p, g.edge_p)
    assert np.array_equal(c.col_idx, g.col_idx) and np.array_equal(c.row_ptr, g.row_ptr)
