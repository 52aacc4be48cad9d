import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 host)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN_DIR, "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def load_golden_graph():
    from relaibilitygpu_gb300 import graphs

    def _load(name):
        return graphs.load_graph(os.path.join(GOLDEN_DIR, "graphs", name + ".txt"))

    return _load


@pytest.fixture(scope="session")
def oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as og  # noqa: E402

    og.lib()
    return og


@pytest.fixture(scope="session")
def engine_lib():
    from relaibilitygpu_gb300 import build, engine

    build.build()
    return engine


def rel_close(a, b, tol=1e-12):
    return abs(a - b) <= tol * max(abs(a), abs(b), 1e-300)
