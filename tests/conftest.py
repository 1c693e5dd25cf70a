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


@pytest.fixture(autouse=True)
def _checked_build_status(request):
    """Against the bounds-checked build (ADVDIFF_LIBRARY=libadvdiff_checked.so), every GPU test
    also requires the device status word to be clear afterwards: an out-of-range index anywhere
    in the test's launches records ADV_ERR_BOUNDS there."""
    yield
    if "checked" not in os.environ.get("ADVDIFF_LIBRARY", "") or request.node.get_closest_marker("gpu") is None:
        return
    from multigpu_advectiondiffusion_gb300 import _native as N
    lib = N.load()
    assert lib.adv_bounds_checked() == 1
    st = lib.adv_device_status(None)
    assert st == N.ADV_OK, f"device status after the test: {N.load().adv_status_string(st)}"
