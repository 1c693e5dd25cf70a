"""The bounds-checked build (libadvdiff_checked.so, ADV_BOUNDS_CHECK): the parity suites of the
stage kernels, the batched kernels and the reference operators run against it in a child process
(ADVDIFF_LIBRARY selects the build); every global-memory index of those kernels, and their
dynamic shared-memory slot indices, is tested before use, and an index out of range would skip
the access and leave ADV_ERR_BOUNDS in the device status word, which tests/conftest.py reads after
every test of the run. Nothing traps or faults: the checks only record."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

from multigpu_advectiondiffusion_gb300 import _native as N

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
SUITES = ["tests/test_gpu_heat.py", "tests/test_gpu_heat2d_multi.py", "tests/test_gpu_heat_twostep.py",
          "tests/test_gpu_burgers.py", "tests/test_gpu_ensemble.py", "tests/test_gpu_reference_kernels.py",
          "tests/test_gpu_compat.py"]


def test_parity_suites_pass_against_the_checked_build(cuda):
    lib = N.LIBDIR / "libadvdiff_checked.so"
    assert lib.exists(), "build() makes libadvdiff_checked.so beside libadvdiff.so"
    env = dict(os.environ, ADVDIFF_LIBRARY="libadvdiff_checked.so")
    r = subprocess.run([sys.executable, "-m", "pytest", *SUITES, "-m", "gpu", "-q", "-x", "-p", "no:cacheprovider",
                        "-k", "not full_size"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=1500)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert " passed" in r.stdout
