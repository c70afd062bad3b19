import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the GB300 kernels)")


@pytest.fixture(scope="session")
def gpu():
    """GPU tests fail (not skip) without a device: a missing GPU must not look like a pass."""
    import torch

    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    return torch.device("cuda:0")
