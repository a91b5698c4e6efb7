import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: long-running test")


@pytest.fixture(scope="session")
def pfft_lib():
    import pfft_gb300
    from pfft_gb300 import build as b
    b.build()
    return pfft_gb300.lib()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch
