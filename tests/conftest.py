import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "graph-cut-ransac_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GPU box)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.load()
    return O


@pytest.fixture(scope="session")
def gcr():
    """The engine's Python entry points; the library must be built (no fallback)."""
    import pygcransac
    pygcransac._abi.load()
    return pygcransac
