import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built native library")


@pytest.fixture(scope="session")
def ff():
    """The package with its native library built (fails loudly if it cannot be)."""
    import __graft_entry__
    __graft_entry__.build()
    import fourierflows.jl_gb300 as m
    return m


@pytest.fixture(scope="session")
def cuda(ff):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    torch.cuda.set_device(0)
    return torch
