import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def golden_movegen():
    d = np.load(os.path.join(HERE, "golden", "movegen_golden.npz"))
    return d["boards"], d["moves"], d["counts"]


@pytest.fixture(scope="session")
def golden_playout():
    return dict(np.load(os.path.join(HERE, "golden", "playout_golden.npz")))


@pytest.fixture(scope="session")
def lib_built():
    """Build libgpuai.so (cross-compiles without a GPU)."""
    from gpu_ai_gb300.build import build
    return build()


@pytest.fixture(scope="session")
def engine(lib_built):
    from gpu_ai_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()
