"""Shared test setup: the `gpu` marker, import paths, and builders for the CUDA library and the
CPU oracle (the oracle is the checker; see oracle/pyoracle.py)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def agb():
    """The built CUDA library; GPU tests fail (not skip) when it or the GPU is missing."""
    from aurora_gb300 import build
    build.build()
    import torch
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    from aurora_gb300 import _abi
    return _abi.library()
