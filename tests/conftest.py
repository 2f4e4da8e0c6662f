import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the native library's kernels")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the native library and the oracle once per session (no-ops when up to date)."""
    from gridcl_gb300 import build as product_build
    from oracle import oracle as orc

    product_build.build()
    orc.build()
    yield


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("a -m gpu test ran without a CUDA device")
    return torch.device("cuda")
