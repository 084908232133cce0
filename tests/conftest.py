import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built CUDA library")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA backend on a machine with a GPU; builds it when missing."""
    from azu_gb300 import _abi, build
    if not os.path.exists(_abi.LIB_PATH):
        build.build()
    import torch
    assert torch.cuda.is_available(), "gpu tests need a CUDA device"
    return _abi.load()
