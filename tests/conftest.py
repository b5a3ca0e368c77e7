import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the kernels through the C ABI")


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree if needed; never a CPU stand-in."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from epic2d_mcc_gb300 import build as B

    B.build()
    import epic2d_mcc_gb300 as E

    return E
