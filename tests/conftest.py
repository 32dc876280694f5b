import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300)")
    config.addinivalue_line("markers", "slow: long CPU test")


def has_gpu() -> bool:
    try:
        import ctypes
        lib = ctypes.CDLL("libcudart.so") if False else None  # noqa: F841
        import torch  # noqa: F401
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def engine():
    from ekgsim_gb300.engine import Engine
    e = Engine(0)
    yield e


REF_ROOT = "/root/reference"


def reference_available() -> bool:
    return os.path.isdir(REF_ROOT)
