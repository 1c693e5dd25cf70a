"""Runs the reference's MATLAB Burgers prototypes here and stores their outputs as fixtures.

Input: the reference checkout (argv[1]). Output: tests/golden/matlab_burgers_prototypes.npz.
The prototype files run unmodified through tests/golden/matlab_subset.py:

* the residual functions Matlab_Prototipes/InviscidBurgersNd/WENO{5,7}resAdv_{X,Y,Z}.m (3D and
  2D fields) and WENO{5,7}resAdv1d.m, on seeded random fields (signs mixed, so both split
  parts matter) and on the drivers' smooth Gaussian;
* the "Solver Loop" sections of LFWENO{5,7}FDM{2,3}d.m, with the drivers' own flux handles,
  CFL and tEnd, on grids smaller than the drivers' 100^d (the only change: nx, ny, nz);
* the 1D drivers LFWENO{5,7}FDM1d.m as they stand, up to their final plot: their own grid,
  CFL, tEnd and initial condition (CommonIC.m case 9, a displaced square jump).

MATLAB arrays are (y, x, z); the fixtures store fields x-fastest as the oracle does
([z][y][x] in numpy). The 2D/3D initial fields are computed here (the drivers' formula
u0 = exp(-(x^2+y^2+z^2)/0.1) on the node grid [-1, 1]^d); every run's u0 is stored with its
results, so a test feeds the same u0 to the oracle. Re-run: python tests/golden/make_weno_golden.py <reference root>
"""
from __future__ import annotations

import hashlib
import re
import os
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from matlab_subset import Interpreter  # noqa: E402

PROTO = Path("Matlab_Prototipes/InviscidBurgersNd")


def to_matlab(a: np.ndarray) -> np.ndarray:
    """x-fastest [z][y][x] / [y][x] / [x] -> MATLAB (y, x, z) / (y, x) / (1, x)."""
    if a.ndim == 3:
        return np.ascontiguousarray(a.transpose(1, 2, 0))
    if a.ndim == 2:
        return a.copy()
    return a.reshape(1, -1).copy()


def from_matlab(m: np.ndarray, ndim: int) -> np.ndarray:
    m = np.asarray(m, dtype=np.float64)
    if ndim == 3:
        return np.ascontiguousarray(m.transpose(2, 0, 1))
    if ndim == 2:
        return m.copy()
    return m.reshape(-1).copy()


def driver_settings(text: str, interp: Interpreter) -> dict:
    """The driver's CFL, tEnd and the 'burgers' flux handles, run from the driver's own lines."""
    env: dict = {}
    lines = text.splitlines()
    for key in ("CFL", "tEnd"):
        line = next(l for l in lines if re.match(rf"\s*{key}\s*=", l))
        interp.run(line, env)
    k = next(i for i, l in enumerate(lines) if re.search(r"case\s+'burgers'", l))
    interp.run("\n".join(lines[k + 1:k + 3]), env)
    assert callable(env["flux"]) and callable(env["dflux"])
    return env


def solver_loop(text: str) -> str:
    m = re.search(r"^%% Solver Loop\s*$(.*?)^%% (?:Final Plot|Post-process)", text, re.S | re.M)
    assert m, "solver loop section not found"
    return m.group(1)


def gaussian(shape_xyz, dx):
    axes = [-1.0 + dx * np.arange(n) for n in shape_xyz]
    if len(shape_xyz) == 3:
        z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
        return 1.0 * np.exp(-(x ** 2 + y ** 2 + z ** 2) / 0.1)
    y, x = np.meshgrid(axes[1], axes[0], indexing="ij")
    return 1.0 * np.exp(-(x ** 2 + y ** 2) / 0.1)


def main(root: Path) -> None:
    pdir = root / PROTO
    interp = Interpreter(pdir)
    out: dict[str, np.ndarray] = {}
    rng = np.random.default_rng(20240607)
    burgers = driver_settings((pdir / "LFWENO7FDM3d.m").read_text(), interp)
    flux, dflux = burgers["flux"], burgers["dflux"]

    # ---- residual functions
    fields = {
        "rand3": rng.standard_normal((7, 8, 9)),          # [z][y][x]: nx=9, ny=8, nz=7
        "smooth3": 0.2 + gaussian((9, 8, 7), 2.0 / 8),     # nx=9, ny=8, nz=7, positive
        "rand2": rng.standard_normal((10, 13)),           # [y][x]: nx=13, ny=10
        "rand1": rng.standard_normal(23),
        "smooth1": np.sin(np.pi * np.linspace(-1, 1, 23)) + 0.3,
    }
    h = {0: 0.11, 1: 0.13, 2: 0.17}
    count = 0
    for name, a in fields.items():
        out[f"res/{name}/u"] = a
        ndim = a.ndim
        for order in (5, 7):
            axes = ["X", "Y", "Z"][:ndim] if ndim > 1 else ["1d"]
            for ax_i, ax in enumerate(axes):
                n_axis = a.shape[::-1][ax_i]
                fn = f"WENO{order}resAdv_{ax}" if ax != "1d" else f"WENO{order}resAdv1d"
                r = interp.call_file(fn, [to_matlab(a), flux, dflux, h[ax_i], float(n_axis)])
                out[f"res/{name}/o{order}/a{ax_i}"] = from_matlab(r, ndim)
                count += 1
    out["res/h"] = np.array([h[0], h[1], h[2]])

    # ---- solver loops of the 2D and 3D drivers on small grids
    runs = {("5", 2): 24, ("7", 2): 24, ("5", 3): 12, ("7", 3): 12}
    for (order, ndim), n in runs.items():
        text = (pdir / f"LFWENO{order}FDM{ndim}d.m").read_text()
        env = driver_settings(text, interp)
        dx = 2.0 / (n - 1)
        u0 = gaussian((n,) * ndim, dx)
        env.update({"u0": to_matlab(u0), "nx": float(n), "ny": float(n), "nz": float(n),
                    "dx": dx, "dy": dx, "dz": dx})
        interp.run(solver_loop(text), env)
        key = f"run/o{order}/d{ndim}"
        out[key + "/u0"] = u0
        out[key + "/u"] = from_matlab(env["u"], ndim)
        out[key + "/t_it_cfl_tend_dx"] = np.array([env["t"], env["it"], env["CFL"], env["tEnd"], dx])

    # ---- the 1D drivers, whole (everything before the final plot)
    for order in ("5", "7"):
        text = (pdir / f"LFWENO{order}FDM1d.m").read_text()
        m = re.search(r"^%% (?:Final Plot|Post-process)", text, re.M)
        env = interp.run(text[:m.start()], {})
        key = f"run/o{order}/d1"
        out[key + "/u0"] = from_matlab(env["u0"], 1)
        out[key + "/u"] = from_matlab(env["u"], 1)
        out[key + "/t_it_cfl_tend_dx"] = np.array([env["t"], env["it"], env["CFL"], env["tEnd"], env["dx"]])

    files = sorted({f"WENO{o}resAdv_{a}.m" for o in (5, 7) for a in "XYZ"} |
                   {f"WENO{o}resAdv1d.m" for o in (5, 7)} | {"CommonIC.m"} |
                   {f"LFWENO{o}FDM{d}d.m" for o in (5, 7) for d in (1, 2, 3)})
    digest = "\n".join(f"{f} {hashlib.sha256((pdir / f).read_bytes()).hexdigest()}" for f in files)
    out["meta/source_sha256"] = np.array(digest)
    out["meta/calls"] = np.array(repr(sorted(interp.calls.items())))
    dst = Path(__file__).resolve().parent / "matlab_burgers_prototypes.npz"
    np.savez_compressed(dst, **out)
    print("wrote", dst, f"({count} residual cases, {len(runs) + 2} solver loops)")
    print(sorted(interp.calls.items()))


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ADV_REFERENCE_DIR", "/root/reference")))
