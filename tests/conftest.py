import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (test infrastructure), built on first use."""
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def native():
    """The bicos_gb300 C ABI, built in-tree on first use."""
    from libbicos_gb300 import _native, build
    build.build()
    return _native


@pytest.fixture(scope="session")
def cuda(native):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    native.load()
    return torch.device("cuda:0")


def golden(name):
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", name), allow_pickle=False)
