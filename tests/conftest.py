import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "inmost-fem_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the anigpu kernels)")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def restated():
    from oracle.oracle import Restated
    return Restated()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(REPO, "tests", "golden", "golden.npz"))


@pytest.fixture(scope="session")
def lib():
    """The anigpu handle; building the library first if it is missing."""
    import anigpu
    if not os.path.exists(anigpu.LIB_PATH):
        anigpu.build()
    if not gpu_available():
        pytest.skip("no CUDA device")
    return anigpu.Anigpu(0)
