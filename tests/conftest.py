import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
for p in (REPO / "wflow.jl_gb300", REPO / "oracle", REPO):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")
    config.addinivalue_line("markers", "slow: long-running parity case")


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """The in-tree CUDA library on a GPU machine; the test fails loudly if it is missing."""
    if not cuda_available():
        pytest.skip("no CUDA device")
    from wflow_gb300 import abi, build
    build.build_all()
    return abi.load_library()
