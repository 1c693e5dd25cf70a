import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")


@pytest.fixture(scope="session")
def native():
    """The product library, built in-tree if needed (nvcc cross-compiles without a GPU)."""
    from multigpu_advectiondiffusion_gb300 import _native
    if not _native.lib_path().exists():
        from multigpu_advectiondiffusion_gb300 import build
        build.build()
    return _native.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def cuda(native):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return torch.device("cuda:0")
