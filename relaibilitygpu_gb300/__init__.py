"""GB300 engine for two-terminal network reliability by path decomposition.

The compute path is CUDA (libnr.so, built for sm_103a); this package holds
the seeded graph generators, the ctypes binding of the C ABI and the build
recipe.
"""
from .graphs import (Graph, batch_instances, complete, format_graph, from_adjacency, from_arcs, from_edges, gnm, grid,
                     load_graph, parse_graph_text, rgg, save_graph)
from .engine import (Batch, Context, MatrixBatch, autotune, options_dict, NrError, Result, initial_mask, lib,
                     load_graph_file, make_options, reliability)

__all__ = [
    "Graph", "batch_instances", "complete", "format_graph", "from_adjacency", "from_arcs", "from_edges", "gnm", "grid",
    "load_graph", "parse_graph_text", "rgg", "save_graph", "Batch", "Context", "MatrixBatch", "autotune", "options_dict", "NrError", "Result", "initial_mask",
    "lib", "load_graph_file", "make_options", "reliability",
]
