import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the product kernels")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def built_oracle():
    from oracle import build

    build.build_oracle()
    return True


@pytest.fixture(scope="session")
def built_lib():
    from elanfmt_gb300 import build

    build.build()
    return True


@pytest.fixture(scope="session")
def cuda_device():
    """The product on a GPU: fails (not skips) when the device or the library is missing."""
    from elanfmt_gb300 import build

    build.build()
    import torch

    assert torch.cuda.is_available(), "GPU test without a CUDA device"
    torch.zeros(1, device="cuda")
    return 0
