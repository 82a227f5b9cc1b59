import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the hand-written kernels")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from md_sim_wolfschwenger_gb300 import build as B
    B.build()
    import oracle
    oracle.build()
    yield
