"""The reference's own single-GPU programs, run unmodified against this library.

Each program's main.cpp + tools.cpp is linked without its kernels.cu against the compatibility
library that exports the same extern "C" names (oracle/ref_build.py: refmain_<name>), then run with
the reference's own command line on small grids:
  * heat 3D and 2D, dense and pitched (SingleGPU/Diffusion3d_baselineCode/main.cpp:106-138,
    SingleGPU/Diffusion{2d,3d}_PitchedMem/main.cpp): their result.bin (WRITE is 1 in their headers)
    equals the oracle's FP64 run rounded to float32 bit for bit, and the PrintSummary block reports
    the oracle's iteration count and final time;
  * Burgers 3D, dense and pitched (SingleGPU/Burgers3d_WENO5/main.cpp:127-161): the printed step
    count and final time equal the oracle's dt loop (its header sets WRITE to 0, so the program
    writes no field; the field itself is compared through the same extern "C" names in
    tests/test_gpu_compat.py);
  * the z-blocked heat program (SingleGPU/Diffusion3d_Blocking/main.cpp:101-144): result.bin
    equals the oracle's restatement of its loop; the shared-memory Burgers program
    (SingleGPU/Burgers3d_WENO5_SharedMem/main.cpp:136-178): step count and final time.
"""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig, HeatConfig

pytestmark = pytest.mark.gpu

REF = Path(__file__).resolve().parent.parent / "oracle" / "_ref"


def _run(name: str, args: list, cwd: Path) -> str:
    exe = REF / f"refmain_{name}"
    if not exe.exists():
        pytest.skip(f"{exe.name} not built (the reference sources were not staged)")
    r = subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, timeout=300, cwd=cwd)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r.stdout


def _field(line: str, out: str) -> str:
    m = re.search(rf"^{re.escape(line)}\s*:\s*(\S+)", out, re.M)
    assert m, (line, out[-1500:])
    return m.group(1)


@pytest.mark.parametrize("name", ["heat3d", "heat3d_pitched"])
@pytest.mark.parametrize("dims,iters", [((33, 33, 33), 20), ((41, 37, 35), 7)])
def test_reference_heat3d_program(cuda, oracle, tmp_path, name, dims, iters):
    nx, ny, nz = dims
    C, L = 1.0, 10
    out = _run(name, [C, L, L, L, nx, ny, nz, iters, 8, 8, 8], tmp_path)
    cfg = HeatConfig.reference_3d(C, L, L, L, nx, ny, nz)
    u0 = oracle.ic_heat_ref(3, nx, ny, nz, L / (nx - 1), L / (ny - 1), L / (nz - 1))
    want = oracle.heat_run(cfg, u0, iters, 1).astype(np.float32)
    got = np.fromfile(tmp_path / "result.bin", dtype=np.float32)
    np.testing.assert_array_equal(got, want)
    assert int(_field("Iterations", out)) == iters
    assert float(_field("Final Time", out)) == pytest.approx(0.1 + cfg.dt * iters, rel=1e-5)


@pytest.mark.parametrize("name", ["heat2d", "heat2d_pitched"])
@pytest.mark.parametrize("dims,iters", [((64, 64), 30), ((101, 77), 9)])
def test_reference_heat2d_program(cuda, oracle, tmp_path, name, dims, iters):
    nx, ny = dims
    C, L = 1.0, 10
    out = _run(name, [C, L, L, nx, ny, iters, 16, 16], tmp_path)
    cfg = HeatConfig.reference_2d(C, L, L, nx, ny)
    u0 = oracle.ic_heat_ref(2, nx, ny, 1, L / (nx - 1), L / (ny - 1), 1.0)
    want = oracle.heat_run(cfg, u0, iters, 1).astype(np.float32)
    got = np.fromfile(tmp_path / "result.bin", dtype=np.float32)
    np.testing.assert_array_equal(got, want)
    assert int(_field("Iterations", out)) == iters
    assert float(_field("Final Time", out)) == pytest.approx(0.1 + cfg.dt * iters, rel=1e-5)


@pytest.mark.parametrize("name", ["burgers3d", "burgers3d_pitched"])
@pytest.mark.parametrize("n,tEnd", [(24, 0.02), (40, 0.05)])
def test_reference_burgers3d_program(cuda, oracle, tmp_path, name, n, tEnd):
    cfl, L = 0.3, 2.0
    out = _run(name, [tEnd, cfl, L, L, L, n, n, n, 8, 8, 8], tmp_path)
    m = re.search(r"dt: (\S+), iterations: (\S+), final time: (\S+)", out)
    assert m, out[-1500:]
    cfg = BurgersConfig.reference(L, L, L, n, n, n, C=1e-5)
    u0 = oracle.ic_burgers_ref(n, n, n, cfg.dx, cfg.dy, cfg.dz)
    _, t_w, it_w = oracle.burgers_run(cfg, u0, tEnd, cfl, 0, C_visc=1e-5, max_steps=1 << 20)
    assert int(float(m.group(2))) == it_w
    assert float(m.group(3)) == pytest.approx(t_w, rel=1e-5)
    assert "Burgers-3D GPU-WENO5" in out


@pytest.mark.parametrize("dims,iters", [((33, 33, 33), 20), ((41, 37, 35), 7)])
def test_reference_heat3d_blocking_program(cuda, oracle, tmp_path, dims, iters):
    nx, ny, nz = dims
    C, L = 1.0, 10
    out = _run("heat3d_blocking", [C, L, L, L, nx, ny, nz, iters], tmp_path)
    cfg = HeatConfig.reference_3d(C, L, L, L, nx, ny, nz)
    u0 = oracle.ic_heat_ref(3, nx, ny, nz, L / (nx - 1), L / (ny - 1), L / (nz - 1))
    want = oracle.heat_blocking_run(nx, ny, nz, cfg.kx, cfg.ky, cfg.kz, cfg.dt, iters, u0).astype(np.float32)
    got = np.fromfile(tmp_path / "result.bin", dtype=np.float32)
    np.testing.assert_array_equal(got, want)
    assert int(_field("Iterations", out)) == iters


@pytest.mark.parametrize("n,tEnd", [(24, 0.02), (40, 0.05)])
def test_reference_burgers3d_sharedmem_program(cuda, oracle, tmp_path, n, tEnd):
    cfl, L = 0.3, 2.0
    out = _run("burgers3d_sharedmem", [tEnd, cfl, L, L, L, n, n, n], tmp_path)
    m = re.search(r"dt: (\S+), iterations: (\S+), final time: (\S+)", out)
    assert m, out[-1500:]
    it_w, t_w = oracle.burgers_ref_steps(tEnd, cfl, L, L, L, n, n, n)
    assert int(float(m.group(2).rstrip(","))) == it_w
    assert float(m.group(3)) == pytest.approx(t_w, rel=1e-5)
    assert "Burgers-3D GPU-WENO5" in out
