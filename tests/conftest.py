import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and runs the native kernels")
    config.addinivalue_line("markers", "slow: full-size cases")


@pytest.fixture(scope="session")
def built_lib():
    """libpanostitch.so built in-tree (nvcc cross-compiles without a GPU)."""
    from panostitcher_gb300 import build as B
    B.build()
    import panostitcher_gb300 as P
    return P.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def cuda(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    torch.cuda.set_device(0)
    return torch
