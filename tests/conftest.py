import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session")
def built_lib():
    """Builds (if stale) and loads libbgemm_gb300.so."""
    import batchgemm_gb300 as bg
    bg.build()
    return bg.lib()


@pytest.fixture(scope="session")
def cuda(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")
