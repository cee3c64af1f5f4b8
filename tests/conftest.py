import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def tklib():
    """libtk_fdk.so, built in-tree if missing (nvcc cross-compiles without a GPU)."""
    from tomokvas_gb300 import _build, _lib

    _build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tomokvas_gb300 import _build

    _build.build()
    torch.cuda.init()
    return torch.device("cuda:0")
