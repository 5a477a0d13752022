import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libfauxglcuda")


@pytest.fixture(scope="session")
def gpu_lib():
    """libfauxglcuda on a GPU: fail loudly if the extension is missing."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a GPU")
    from fauxgl_gb300 import _abi

    lib_path = _abi.LIB_PATH
    if not os.path.exists(lib_path):
        pytest.fail("libfauxglcuda.so is not built; run __graft_entry__.build()")
    torch.cuda.set_device(0)
    return _abi.load_library()
