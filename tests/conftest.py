import importlib
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def po():
    """The CPU oracle (test infrastructure), built on first use."""
    from oracle import pyoracle

    pyoracle.build(ref=False)
    return pyoracle


@pytest.fixture(scope="session")
def chy():
    """The product package (ctypes over libchybrid.so)."""
    return importlib.import_module("collisional-hybrid_gb300")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(os.path.join(REPO, "tests", "golden", "reference_golden.npz"))


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
