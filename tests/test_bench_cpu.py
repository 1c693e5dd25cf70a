"""The benchmark's CPU legs (no GPU): the tuned CPU loop behind the CPU baseline (equal to the oracle
bit for bit), its rate on all host threads and on one thread with the host CPU named, and the
`--impl reference` line (the path's CPU restatement on the host cores, same config as the GPU arm,
the library itself never loaded)."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402
from multigpu_advectiondiffusion_gb300.solvers import HeatConfig  # noqa: E402


@pytest.mark.parametrize("ndim,n,steps", [(3, 37, 7), (3, 40, 8), (2, 301, 9), (2, 64, 6)])
def test_tuned_cpu_loop_equals_the_oracle(oracle, ndim, n, steps):
    """The CPU baseline's loop (two buffers, branch-free interior, separate boundary pass) gives
    the oracle's FP32 forward-Euler result in the reference's operand order bit for bit, for even
    and odd step counts."""
    cfg = HeatConfig.dirichlet_o2(ndim, n)
    u0 = (oracle.ic_heat3d_blobs(n, n, n, 2) if ndim == 3 else oracle.ic_heat2d_gauss_noise(n, n, 1, 1e-3))
    u0 = u0.astype(np.float32)
    want = oracle.heat_run(cfg, u0, steps, 0, fp32_order="reference")
    np.testing.assert_array_equal(oracle.cpu_heat_euler_o2(cfg, u0.copy(), steps), want)


def test_tuned_cpu_loop_keeps_frozen_layers(oracle):
    """Frozen layers deeper than the stencil radius are copied through, only the outermost zeroed."""
    cfg = HeatConfig.dirichlet_o2(3, 20)
    cfg.frozen = 3
    u0 = np.random.default_rng(1).random(20 ** 3).astype(np.float32)
    want = oracle.heat_run(cfg, u0, 3, 0, fp32_order="reference")
    np.testing.assert_array_equal(oracle.cpu_heat_euler_o2(cfg, u0.copy(), 3), want)


def test_cpu_baseline_reports_all_cores_one_core_and_model():
    cfg = HeatConfig.dirichlet_o2(3, 32)
    u0 = bench.ic_heat3d_blobs(32, 32, 32, 2, source="oracle").astype(np.float32)
    cpu = bench.cpu_baseline_heat(cfg, u0, 2000, 0.2)
    assert cpu["kind"] == "port" and cpu["unit"] == "Gcell-updates/s"
    assert cpu["value"] > 0 and cpu["one_core_value"] > 0
    assert cpu["cores"] >= 1 and "32^3" in cpu["sample"] and "tuned CPU loop" in cpu["sample"]
    assert isinstance(cpu["cpu_model"], str) and cpu["cpu_model"]


def _reference_line(workload: str) -> dict:
    """Runs `bench.py --impl reference` in a child process that reports which shared objects it
    mapped, and returns its JSON line with those paths under "_maps"."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3', "
            f"'--workload', '{workload}']; runpy.run_path('bench.py', run_name='__main__'); "
            "print('MAPS', sorted({l.split()[-1] for l in open('/proc/self/maps') if l.rstrip().endswith('.so') "
            "or '.so.' in l.split()[-1]}))")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    maps = [ln for ln in r.stdout.splitlines() if ln.startswith("MAPS")]
    line["_maps"] = maps[0] if maps else ""
    return line


def test_reference_arm_prints_one_contract_line_without_loading_the_library():
    """`bench.py --impl reference` (the tuned CPU loop on the host cores) prints one JSON line with
    the contract's fields, a measured ms_per_step, the GPU arm's config, and never maps
    libadvdiff.so (its inputs come from the oracle's generators); it needs no GPU."""
    line = _reference_line("heat3d")
    assert line["impl"] == "reference" and line["metric"] == "Gcell-updates/s/RK-stage"
    assert line["value"] > 0 and line["unit"] == "Gcell-updates/s" and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["config"] == bench.heat_config("heat3d", 1)
    assert line["ms_per_step"] > 0
    cpu = line["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and cpu["value"] == line["value"] and cpu["cpu_model"]
    assert line["e2e"] == {"value": line["value"], "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert "liboracle.so" in line["_maps"] and "libadvdiff" not in line["_maps"]


def test_reference_arm_heat2d_samples_the_plain_method():
    """C1 (2D 512^2, 1000 steps, the plain method): up to the whole solve per step within the CPU
    budget (all 1000 steps on an idle 16-core host)."""
    line = _reference_line("heat2d")
    assert line["config"] == bench.heat_config("heat2d", 1)
    assert "of the 1000 time steps" in line["cpu_baseline"]["sample"]
    assert "libadvdiff" not in line["_maps"]
