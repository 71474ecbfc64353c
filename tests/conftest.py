import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through libmumag_cuda's C-ABI")


def pytest_sessionstart(session):
    # the CPU tests call the library's host-only setup entry points: build it when missing
    from mumag_matrixfree2_gb300 import build

    build.build()


@pytest.fixture(scope="session")
def cuda_ok():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("a gpu-marked test ran without a CUDA device")
    return True
