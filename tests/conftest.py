import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle():
    """The C restatement of the reference (test checker only)."""
    from oracle import build, pyoracle
    build.build_port()
    return pyoracle


@pytest.fixture(scope="session")
def gpu():
    """The CUDA library, loaded through its C ABI; fails loudly without a GPU."""
    from opentissue_gb300 import build, capi
    build.build()
    lib = capi.lib()
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test on a machine without a CUDA device")
    torch.cuda.init()
    return lib
