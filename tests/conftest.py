import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build(ref=False)
    return O


@pytest.fixture(scope="session")
def gpulib():
    """The built CUDA library; GPU tests fail loudly if it is missing."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for gpu-marked tests")
    from ffea_gb300 import build as B
    B.build()
    from ffea_gb300 import _lib as L
    return L.lib()


@pytest.fixture(scope="session")
def gpulib_cpu():
    """The built library for its host-only entry points (no GPU needed)."""
    from ffea_gb300 import build as B
    B.build()
    from ffea_gb300 import _lib as L
    return L.lib()
