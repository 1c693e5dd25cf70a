"""The benchmark's CPU-baseline leg (no GPU): the oracle's heat rate on all host threads and on
one thread, with the host CPU named, as bench.py reports it beside the GPU numbers."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import bench  # noqa: E402
from multigpu_advectiondiffusion_gb300.solvers import HeatConfig  # noqa: E402


def test_cpu_baseline_reports_all_cores_one_core_and_model():
    cfg = HeatConfig.dirichlet_o2(3, 32)
    u0 = bench.ic_heat3d_blobs(32, 32, 32, 2).astype(np.float32)
    cpu = bench.cpu_baseline_heat(cfg, u0, 0.2)
    assert cpu["kind"] == "port" and cpu["unit"] == "Gcell-updates/s"
    assert cpu["value"] > 0 and cpu["one_core_value"] > 0
    assert cpu["cores"] >= 1 and "32^3" in cpu["sample"]
    assert isinstance(cpu["cpu_model"], str) and cpu["cpu_model"]
