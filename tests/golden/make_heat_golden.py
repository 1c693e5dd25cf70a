"""Runs the reference's MATLAB heat accuracy study here and stores its numbers as a fixture.

Input: the reference checkout (argv[1]). Output: tests/golden/matlab_heat_accuracy.json.
The functions Matlab_Prototipes/DiffusionNd/diffusion{1,2,3}dTest.m (O4 Laplacian of
Laplace{1,2,3}d.m, SSP-RK3, Dirichlet reset after each step, the dt trim after the step) run
unmodified through tests/golden/matlab_subset.py with tFinal = 1.0 and factor 0.9, the settings
of the recorded TestingAccuracy.log, at the grids the interpreter finishes in about a minute:
nc = 10, 20, 40, 80 in 1D, 10, 20, 40 in 2D, 10 and 20 in 3D. Each case keeps L1, L2, Linf (as
the functions compute them) and the step count. Re-run:
python tests/golden/make_heat_golden.py <reference root>
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))
from matlab_subset import Interpreter  # noqa: E402

PROTO = Path("Matlab_Prototipes/DiffusionNd")
CASES = [(1, 10), (1, 20), (1, 40), (1, 80), (2, 10), (2, 20), (2, 40), (3, 10), (3, 20)]
T_FINAL, FACTOR = 1.0, 0.9


def main(root: Path) -> None:
    pdir = root / PROTO
    interp = Interpreter(pdir)
    runs = []
    for dim, nc in CASES:
        env: dict = {}
        grid = [float(nc)] * dim
        l1, linf = interp.call_file(f"diffusion{dim}dTest", grid + [T_FINAL, FACTOR], nargout=2, env_out=env)
        runs.append({"dim": dim, "nc": nc, "L1": float(l1), "L2": float(env["L2"]), "Linf": float(linf),
                     "steps": int(env["it"])})
        print(runs[-1], flush=True)
    files = sorted([f"diffusion{d}dTest.m" for d in (1, 2, 3)] + [f"Laplace{d}d.m" for d in (1, 2, 3)])
    out = {
        "source": "Matlab_Prototipes/DiffusionNd, run through tests/golden/matlab_subset.py",
        "tFinal": T_FINAL, "factor": FACTOR,
        "source_sha256": {f: hashlib.sha256((pdir / f).read_bytes()).hexdigest() for f in files},
        "calls": dict(sorted(interp.calls.items())),
        "runs": runs,
    }
    dst = Path(__file__).resolve().parent / "matlab_heat_accuracy.json"
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", dst)


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ADV_REFERENCE_DIR", "/root/reference")))
