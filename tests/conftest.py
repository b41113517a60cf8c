import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def orc():
    """The CPU restatement (built on demand)."""
    from oracle import oracle
    if not oracle.available():
        oracle.build()
    return oracle


@pytest.fixture(scope="session")
def kg():
    """The CUDA library through its Python mirror (built on demand)."""
    from kodama_gb300 import build as kbuild
    kbuild.build()
    import kodama_gb300
    return kodama_gb300
