import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _checkers_built():
    from oracle import build as ob
    ob.build_oracle()
    ob.build_ref()


@pytest.fixture(scope="session")
def gpu_lib():
    """The native library, built for sm_103a; a GPU test fails (not skips)
    when it cannot be loaded."""
    import torch
    assert torch.cuda.is_available(), "GPU test needs CUDA"
    from tmr_gb300 import build
    build.build()
    from tmr_gb300 import _lib
    return _lib.lib()
