import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300)")
    config.addinivalue_line("markers", "slow: long CPU test")


@pytest.fixture(scope="session")
def engine():
    from ekgsim_gb300.engine import Engine
    e = Engine(0)
    yield e


def reference_dir():
    """Sources of the reference simulator, when present: $EKGSIM_REFERENCE, else a checkout named
    ``reference`` beside this repository; None when neither exists (as on the GPU machines)."""
    from oracle.refpath import reference_dir as rd
    return rd()
