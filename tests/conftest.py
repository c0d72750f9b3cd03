import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def built_lib():
    """Build libgbspmm.so if needed (nvcc cross-compiles without a GPU)."""
    from spmm_eval_gb300 import build as b
    return b.build()


@pytest.fixture(scope="session")
def cuda(built_lib):
    """A GPU test never skips silently: no device is a failure."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected but torch.cuda.is_available() is False")
    torch.cuda.init()
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.lib()
    return oracle
