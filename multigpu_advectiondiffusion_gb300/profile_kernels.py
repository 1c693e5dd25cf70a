"""Direct launches of one hot kernel for profilers (ncu): no CUDA graph, no host loop logic.

    python -m multigpu_advectiondiffusion_gb300.profile_kernels heat3d   [--n 256] [--launches 6]
    python -m multigpu_advectiondiffusion_gb300.profile_kernels heat3d2  [--n 256] [--launches 6]
    python -m multigpu_advectiondiffusion_gb300.profile_kernels burgers3d [--n 256] [--launches 4]
    python -m multigpu_advectiondiffusion_gb300.profile_kernels weno7    [--n 256] [--launches 2]

heat3d: the 3D O2 forward-Euler stage on an n^3 FP32 grid (ping-pong between two buffers).
heat3d2: the same problem through adv_heat_run, whose launches each advance two Euler steps
(2 x launches time steps).
burgers3d: the periodic WENO5-Z global-Lax-Friedrichs SSP-RK3 stage 1 on an n^3 FP32 grid.
weno7: the WENO7 prototype scheme's right-hand side (adv_weno7_rhs: a face and a residual kernel
per axis) on the prototype's Gaussian at n^3 FP32.
Inputs are the seeded initial conditions of the benchmark workloads, generated on the host.
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("kernel", choices=["heat3d", "heat3d2", "burgers3d", "weno7"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--launches", type=int, default=6)
    ap.add_argument("--dtype", default="f32", choices=["f32", "f64"])
    ap.add_argument("--div", default="fast", choices=["fast", "f32", "f64"])
    a = ap.parse_args(argv)
    import torch

    from . import _native as N
    from .solvers import BurgersConfig, HeatConfig, burgers_stage, heat_run, heat_stage

    dev = torch.device("cuda:0")
    lib = N.load()
    npdt = np.float32 if a.dtype == "f32" else np.float64
    n = a.n
    if a.kernel == "heat3d2":
        cfg = HeatConfig.dirichlet_o2(3, n)
        u0 = np.empty(n ** 3)
        N.check(lib.adv_ic_heat3d_blobs(n, n, n, 2, 8, u0.ctypes.data_as(N.C.POINTER(N.C.c_double))), "ic")
        u = torch.from_numpy(u0.astype(npdt)).to(dev)
        heat_run(cfg, u, 2 * a.launches)
    elif a.kernel == "heat3d":
        cfg = HeatConfig.dirichlet_o2(3, n)
        u0 = np.empty(n ** 3)
        N.check(lib.adv_ic_heat3d_blobs(n, n, n, 2, 8, u0.ctypes.data_as(N.C.POINTER(N.C.c_double))), "ic")
        u = torch.from_numpy(u0.astype(npdt)).to(dev)
        v = torch.empty_like(u)
        for _ in range(a.launches):
            heat_stage(cfg, 1, u, u, v)
            u, v = v, u
    elif a.kernel == "weno7":
        from .solvers import Weno7Config, weno7_rhs, weno7_workspace
        x = np.linspace(-1.0, 1.0, n)
        z, y, xx = np.meshgrid(x, x, x, indexing="ij")
        u = torch.from_numpy(np.exp(-(xx ** 2 + y ** 2 + z ** 2) / 0.1).astype(npdt).ravel()).to(dev)
        h = 2.0 / (n - 1)
        cfg = Weno7Config(n, n, n, h, h, h)
        L = torch.empty_like(u)
        ws = weno7_workspace(cfg, u)
        for _ in range(a.launches):
            weno7_rhs(cfg, u, L, ws)
    else:
        cfg = BurgersConfig.periodic(n, weno="z", div=a.div)
        u0 = np.empty(n ** 3)
        N.check(lib.adv_ic_burgers_fourier(n, n, n, 2.0, 3, 16, 0.1, u0.ctypes.data_as(N.C.POINTER(N.C.c_double))),
                "ic")
        u = torch.from_numpy(u0.astype(npdt)).to(dev)
        v = torch.empty_like(u)
        alpha = float(np.abs(u0).max())
        for _ in range(a.launches):
            burgers_stage(cfg, 1, u, u, v, 1e-3, alpha)
    torch.cuda.synchronize()
    print(f"{a.kernel} n={n} {a.dtype}: {a.launches} launches ok")


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    main()
