import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libspgemm_gb300.so")


@pytest.fixture(scope="session")
def handle():
    """One library handle for the GPU tests (fails loudly if the library is missing)."""
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from gpu_spgemm_gb300 import api
    with api.Handle(0) as h:
        yield h
