"""The command-line drivers end to end (the reference's argv, result.bin) and their snapshots:
a run stopped after some steps with --checkpoint and continued with --restart ends bit for bit
where the uninterrupted run ends, with the same step count."""
import re
import subprocess

import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import HeatConfig

pytestmark = pytest.mark.gpu


def _run(args, cwd):
    r = subprocess.run([str(N.LIBDIR / args[0]), *map(str, args[1:])], capture_output=True, text=True, cwd=cwd,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_heat3d_driver_equals_oracle_and_resumes_exactly(cuda, native, oracle, tmp_path):
    base = ["heat3d", 1.0, 10, 10, 10, 41, 39, 37]
    _run(base + [30, "--write=1", "--out=full.bin"], tmp_path)
    cfg = HeatConfig.reference_3d(1.0, 10, 10, 10, 41, 39, 37)
    u0 = np.empty(cfg.numel)
    N.check(native.adv_ic_heat_ref(3, 41, 39, 37, 10 / 40, 10 / 38, 10 / 36, u0.ctypes.data_as(N.C.POINTER(N.C.c_double))),
            "ic")
    want = oracle.heat_run(cfg, u0, 30, N.ADV_SSPRK3).astype(np.float32)
    full = np.fromfile(tmp_path / "full.bin", dtype=np.float32)
    np.testing.assert_array_equal(full, want)
    _run(base + [12, "--write=0", "--checkpoint=part.state"], tmp_path)
    out = _run(base + [30, "--write=1", "--out=resumed.bin", "--restart=part.state"], tmp_path)
    assert "restarted from part.state at step 12" in out
    np.testing.assert_array_equal(np.fromfile(tmp_path / "resumed.bin", dtype=np.float32), full)


@pytest.mark.parametrize("flags,n", [
    ([], 40),  # the reference scheme: frozen layers, local LF, viscous, fixed dt, FP64
    (["--bc=periodic", "--lf=global", "--dt=maxu", "--precision=f32", "--ic=fourier", "--div=f64"], 32),
])
def test_burgers3d_driver_resumes_exactly(cuda, native, tmp_path, flags, n):
    base = ["burgers3d"]
    tail = [0.30, 2, 2, 2, n, n, n, *flags]
    out_full = _run(base + [0.12] + tail + ["--write=1", "--out=full.bin", "--checkpoint=full.state"], tmp_path)
    # stop after 4 steps (stopping at a time off the step grid would trim the last step there)
    _run(base + [0.12] + tail + ["--max-steps=4", "--checkpoint=part.state"], tmp_path)
    out_res = _run(base + [0.12] + tail + ["--write=1", "--out=resumed.bin", "--restart=part.state",
                                           "--checkpoint=resumed.state"], tmp_path)
    it = lambda s: int(re.search(r"iterations: (\d+)", s).group(1))
    assert it(out_res) == it(out_full)
    a = np.fromfile(tmp_path / "full.bin", dtype=np.float32)
    b = np.fromfile(tmp_path / "resumed.bin", dtype=np.float32)
    np.testing.assert_array_equal(a, b)
    # the snapshots carry the state in its own precision, the step count and the time
    ha, hb = N.CheckpointHeader(), N.CheckpointHeader()
    assert native.adv_checkpoint_load(str(tmp_path / "full.state").encode(), N.C.byref(ha), None, 0) == N.ADV_OK
    assert native.adv_checkpoint_load(str(tmp_path / "resumed.state").encode(), N.C.byref(hb), None, 0) == N.ADV_OK
    assert (ha.step, ha.t, ha.payload_crc32) == (hb.step, hb.t, hb.payload_crc32)
    assert ha.t == pytest.approx(0.12)


def test_burgers2d_driver_equals_oracle_and_resumes_exactly(cuda, native, oracle, tmp_path):
    """burgers2d with the reference's 2D argv (tEnd CFL L W NX NY bx by): WENO5-JS, local LF,
    dt = CFL dx, its centred Gaussian IC; result.bin equals the FP64 oracle's run, and a run
    stopped after 5 steps and continued ends on the same bits."""
    from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig
    nx, ny = 61, 47
    base = ["burgers2d", 0.1, 0.3, 2, 2, nx, ny, 16, 16]
    out = _run(base + ["--write=1", "--out=full.bin"], tmp_path)
    cfg = BurgersConfig.reference_2d(2.0, 2.0, nx, ny)
    u0 = np.empty(nx * ny)
    N.check(native.adv_ic_burgers_ref2d(nx, ny, cfg.dx, cfg.dy, u0.ctypes.data_as(N.C.POINTER(N.C.c_double))), "ic")
    want, _, it_w = oracle.burgers_run(cfg, u0, 0.1, 0.3, 0)
    assert int(re.search(r"iterations: (\d+)", out).group(1)) == it_w
    full = np.fromfile(tmp_path / "full.bin", dtype=np.float32)
    np.testing.assert_array_equal(full, want.astype(np.float32))
    _run(base + ["--max-steps=5", "--checkpoint=part.state"], tmp_path)
    _run(base + ["--write=1", "--out=resumed.bin", "--restart=part.state"], tmp_path)
    np.testing.assert_array_equal(np.fromfile(tmp_path / "resumed.bin", dtype=np.float32), full)
