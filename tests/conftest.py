import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running full-size case")


@pytest.fixture(scope="session")
def gpu_lib():
    """Loads the in-tree CUDA library (building it first if needed) and
    fails -- never skips -- when it cannot be loaded on a GPU machine."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without CUDA")
    import mini_mdft_gb300 as M
    from mini_mdft_gb300 import build as B
    B.build()
    M.lib()
    return M
