import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library; GPU tests fail loudly (not skip) when it is
    missing, so a silent fallback cannot pass them."""
    if not has_gpu():
        pytest.skip("no CUDA device")
    import nlsemagic_gb300 as ng
    return ng.load()
