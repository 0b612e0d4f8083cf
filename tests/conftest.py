import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library (built here if missing); GPU tests fail loudly without it."""
    from light_garden_gb300 import abi, build
    build.build()
    return abi.load()


@pytest.fixture(scope="session")
def gpu(cuda_lib):
    if not _has_gpu():
        pytest.fail("gpu test collected on a machine without a CUDA GPU")
    return cuda_lib


@pytest.fixture()
def ctx(gpu):
    from light_garden_gb300.runtime import Context
    c = Context()
    yield c
    c.close()
