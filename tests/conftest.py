import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine's kernels)")


@pytest.fixture(scope="session")
def lib():
    """The engine library, built in-tree if needed (no GPU needed to build or load)."""
    from puncpp_gb300 import build_lib, _lib
    build_lib.build()
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as O
    O.build()
    return O
