"""Test configuration: the ``gpu`` marker, import paths, shared fixtures.

``-m "not gpu"`` runs everywhere (oracle vs the reference's known answers,
host logic, the C ABI's exports); ``-m gpu`` needs a CUDA device and calls
the library through its C ABI."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "graph-tool-rs_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gtc():
    """The built library's Python binding (builds libgtc.so if needed)."""
    import build as B  # graph-tool-rs_gb300/build.py
    B.build()
    import graph_tool
    from graph_tool import _ffi
    _ffi.lib()
    return graph_tool
