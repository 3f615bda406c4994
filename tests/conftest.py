import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gsap_lib():
    """libgsap.so, built in-tree if missing (nvcc cross-compiles without a GPU)."""
    from gsap_gb300 import build as b
    b.build()
    from gsap_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def cuda(gsap_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")
