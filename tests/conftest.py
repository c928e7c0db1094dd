import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def cuda():
    """GPU tests fail (not skip) without a device: a silent skip would hide a broken box."""
    import torch
    assert torch.cuda.is_available(), "GPU test collected on a machine without CUDA"
    from bskit_gb300 import _lib
    _lib.load()
    return torch.device("cuda", 0)
