import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
# the reference prints progress by default; keep test output quiet
os.environ.setdefault("PARRSB_VERBOSE_LEVEL", "0")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def lib():
    """The CUDA library, built in-tree if needed (nvcc cross-compiles)."""
    import parrsb_gb300 as P
    return P.library(build_if_missing=True)
