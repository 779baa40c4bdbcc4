import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")


def gpu_available():
    try:
        import torch  # noqa: F401  (only used to ask whether a device exists)
        return torch.cuda.is_available()
    except Exception:
        return os.path.exists("/dev/nvidia0")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    return O
