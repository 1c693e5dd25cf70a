"""Extracts the reference's recorded numbers into tests/golden/reference_pins.json.

Reads, as text only, the files of the reference checkout given as argv[1]:
  * Matlab_Prototipes/DiffusionNd/TestingAccuracy.log -- per-run L1/L2/Linf of the O4 + SSP-RK3
    heat accuracy study (runs in the order 1D, 2D, 3D for each resolution);
  * SingleGPU/*/Run.m header blocks -- grid sizes, iteration counts and "Final Time" values
    printed by the reference drivers, with the command lines of the matching run.sh.
Nothing here executes reference code. Re-run: python tests/golden/make_golden.py <reference root>
"""
from __future__ import annotations

import json
import re
import os
import sys
from pathlib import Path


def accuracy_runs(log: Path):
    txt = log.read_text()
    l1 = [float(x) for x in re.findall(r"L_1 norm: ([0-9.e+-]+)", txt)]
    l2 = [float(x) for x in re.findall(r"L_2 norm: ([0-9.e+-]+)", txt)]
    li = [float(x) for x in re.findall(r"L_inf norm: ([0-9.e+-]+)", txt)]
    assert len(l1) == len(l2) == len(li) == 12, "expected 4 resolutions x 3 dimensions"
    runs = []
    for n in range(4):          # resolution index
        for d in range(3):      # 1D, 2D, 3D
            k = 3 * n + d
            runs.append({"dim": d + 1, "res_index": n, "L1": l1[k], "L2": l2[k], "Linf": li[k]})
    # the summary table's element counts (nE column) for the four resolutions
    ne = sorted({int(x) for x in re.findall(r"^\s*(\d+)\s+\t", txt, flags=re.M)})
    return runs, ne


def run_blocks(runm: Path):
    txt = runm.read_text()
    blocks = []
    for b in re.split(r"% =+ ?[^=\n]+ ?=+\n", txt)[1:]:
        g3 = re.search(r"3D Grid Size\s*:\s*(\d+) x (\d+) x (\d+)", b)
        g2 = re.search(r"2D Grid Size\s*:\s*(\d+) x (\d+)", b)
        it = re.search(r"Iterations\s*:\s*(\d+)", b)
        ft = re.search(r"Final Time\s*:\s*([0-9.e+-]+)", b)
        kt = re.search(r"Kernel time ex. data transfers\s*:\s*([0-9.]+)", b)
        dth = re.search(r"Data transfer\(s\) DtH\s*:\s*([0-9.]+)", b)
        if not it:
            continue
        grid = [int(x) for x in (g3 or g2).groups()]
        blocks.append({"grid": grid, "iterations": int(it.group(1)),
                       "final_time": float(ft.group(1)) if ft else None,
                       "kernel_seconds": float(kt.group(1)) if kt else None,
                       "dth_seconds": float(dth.group(1)) if dth else None})
    return blocks


def main(root: Path) -> None:
    runs, ne = accuracy_runs(root / "Matlab_Prototipes/DiffusionNd/TestingAccuracy.log")
    out = {
        "source": "wme7/MultiGPU_AdvectionDiffusion (text of logs and Run.m headers)",
        "testing_accuracy": {
            "file": "Matlab_Prototipes/DiffusionNd/TestingAccuracy.log",
            "elements": ne,
            "note": "runs reproduce with nc = elements, tEnd = 1.0, factor 0.9 (the .m file's "
                    "nc/tEnd were edited after the log was written)",
            "runs": runs,
        },
        "drivers": {},
    }
    for runm in sorted((root / "SingleGPU").glob("*/Run.m")):
        sh = runm.parent / "run.sh"
        cmd = [l for l in sh.read_text().splitlines() if l.startswith("./")] if sh.exists() else []
        out["drivers"][runm.parent.name] = {"run_sh": cmd[0] if cmd else None, "blocks": run_blocks(runm)}
    dst = Path(__file__).resolve().parent / "reference_pins.json"
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", dst)


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ADV_REFERENCE_DIR", "/root/reference")))
