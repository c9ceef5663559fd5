import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libpog.so")
    config.addinivalue_line("markers", "slow: longer GPU parity runs")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from pour_over_coffee_lbm_gb300 import _lib
    _lib.load()
    return torch.device("cuda")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.load()
    return oracle
