import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gbx():
    """The C-ABI library, built in-tree if needed."""
    from ttg_gb300 import build as b
    import ttg_gb300
    if not os.path.exists(ttg_gb300.LIB_PATH):
        b.build()
    ttg_gb300.lib()
    return ttg_gb300


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    return torch.device("cuda:0")
