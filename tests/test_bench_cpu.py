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


def test_reference_arm_prints_one_contract_line():
    """`bench.py --impl reference` (the oracle on the host cores) prints one JSON line with the
    fields the driver reads; it needs no GPU."""
    import json
    import subprocess
    root = Path(__file__).resolve().parent.parent
    r = subprocess.run([sys.executable, str(root / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["metric"] == "Gcell-updates/s/RK-stage"
    assert line["value"] > 0 and line["unit"] == "Gcell-updates/s" and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["config"]["workload"].startswith("heat3d 256^3")
    cpu = line["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and cpu["value"] == line["value"] and cpu["cpu_model"]
    assert line["e2e"] == {"value": line["value"], "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
