import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def olib():
    import oracle
    return oracle.lib()


@pytest.fixture(scope="session")
def rlib():
    import oracle
    r = oracle.ref_lib()
    if r is None:
        pytest.skip("reference sources not present (reference build unavailable)")
    return r


@pytest.fixture(scope="session")
def gpu():
    """The GPU library; GPU tests fail loudly if it cannot be loaded."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xavs2_gb300
    return xavs2_gb300.load()
