"""The seventh-order WENO prototype solver on the GPU (adv_weno7_rhs / adv_weno7_run).

FP64 is held bit for bit against the reference's own MATLAB prototypes -- the outputs of
Matlab_Prototipes/InviscidBurgersNd/WENO7resAdv_{X,Y,Z}.m and the solver loops of
LFWENO7FDM{2,3}d.m, run through tests/golden/matlab_subset.py into
tests/golden/matlab_burgers_prototypes.npz -- and against the CPU oracle's restatement of them on
other grids; FP32 (a form of its own, written for speed) to stated relative L2 bounds against
FP64.
"""
from pathlib import Path

import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300.solvers import Weno7Config, weno7_rhs, weno7_run

pytestmark = pytest.mark.gpu

FIX = Path(__file__).resolve().parent / "golden" / "matlab_burgers_prototypes.npz"


def _t(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def _cfg(u, h):
    s = u.shape[::-1]
    nx, ny, nz = s[0], s[1], (s[2] if len(s) > 2 else 1)
    hh = list(h) + [1.0] * (3 - len(h))
    return Weno7Config(nx, ny, nz, *hh)


@pytest.mark.parametrize("name", ["rand3", "smooth3", "rand2"])
def test_weno7_rhs_equals_matlab_prototype(cuda, name):
    """The summed residuals equal the prototypes' per-axis residuals summed in axis order."""
    import torch
    fx = np.load(FIX)
    u = fx[f"res/{name}/u"]
    h = fx["res/h"][: u.ndim]
    want = fx[f"res/{name}/o7/a0"]
    for ax in range(1, u.ndim):
        want = want + fx[f"res/{name}/o7/a{ax}"]
    cfg = _cfg(u, h)
    a = _t(u.ravel(), cuda)
    L = torch.full_like(a, float("nan"))
    weno7_rhs(cfg, a, L)
    np.testing.assert_array_equal(L.cpu().numpy().reshape(u.shape), want)


@pytest.mark.parametrize("ndim", [2, 3])
def test_weno7_run_equals_matlab_prototype(cuda, ndim):
    """LFWENO7FDM{2,3}d.m's solver loop (their CFL 0.4, tEnd 0.4) from the fixture's initial state:
    the same step count, end time and field, bit for bit."""
    fx = np.load(FIX)
    k = f"run/o7/d{ndim}"
    t_ref, it_ref, cfl, tend, dx = fx[k + "/t_it_cfl_tend_dx"]
    u0 = fx[k + "/u0"]
    cfg = _cfg(u0, [dx] * ndim)
    a = _t(u0.ravel(), cuda)
    t, it = weno7_run(cfg, a, float(tend), float(cfl))
    assert it == int(it_ref) and t == t_ref
    np.testing.assert_array_equal(a.cpu().numpy().reshape(u0.shape), fx[k + "/u"])


@pytest.mark.parametrize("shape", [(11, 17, 13), (40, 9, 6), (64, 48), (33, 5)])
def test_weno7_rhs_and_run_equal_the_oracle(cuda, oracle, shape):
    """Other grids, ragged and thin (lines shorter than the stencil clamp on both ends)."""
    import torch
    rng = np.random.default_rng(sum(shape))
    u0 = rng.standard_normal(shape[::-1]) * 0.5 + 0.3
    h = [2.0 / (n - 1) for n in shape]
    want = oracle.proto_residual(7, 0, u0, h[0])
    for ax in range(1, len(shape)):
        want = want + oracle.proto_residual(7, ax, u0, h[ax])
    cfg = _cfg(u0, h)
    a = _t(u0.ravel(), cuda)
    L = torch.empty_like(a)
    weno7_rhs(cfg, a, L)
    np.testing.assert_array_equal(L.cpu().numpy().reshape(u0.shape), want)
    uw, tw, itw = oracle.proto_run(7, u0, h, 0.4, 0.05)
    t, it = weno7_run(cfg, a, 0.05, 0.4)
    assert (it, t) == (itw, tw)
    np.testing.assert_array_equal(a.cpu().numpy().reshape(u0.shape), uw)


@pytest.mark.parametrize("shape", [(11, 17, 13), (40, 9, 6), (64, 48), (33, 5), (70, 35, 37), (300, 3), (5, 70, 40)])
def test_weno7_fp32_rhs_within_bound_of_fp64(cuda, oracle, shape):
    """The FP32 state's tiled face kernels (split parts staged once per tile, both parts of a face
    in paired instructions, weights from r_k = e_min / e_k): ragged tiles along every axis, lines
    shorter than the stencil, several tiles per line; relative L2 error of the summed residuals
    against the FP64 oracle <= 5e-6 (a float32 emulation of the form on the host measured 2e-7)."""
    import torch
    rng = np.random.default_rng(sum(shape) + 1)
    u0 = rng.standard_normal(shape[::-1]) * 0.5 + 0.3
    h = [2.0 / (n - 1) for n in shape]
    want = oracle.proto_residual(7, 0, u0, h[0])
    for ax in range(1, len(shape)):
        want = want + oracle.proto_residual(7, ax, u0, h[ax])
    cfg = _cfg(u0, h)
    a = _t(u0.astype(np.float32).ravel(), cuda)
    L = torch.full_like(a, float("nan"))
    weno7_rhs(cfg, a, L)
    got = L.cpu().numpy().astype(np.float64).reshape(u0.shape)
    assert np.isfinite(got).all()
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert rel <= 5e-6, rel


def test_weno7_fp32_run_within_bound_of_fp64(cuda, oracle):
    """FP32 state, 48^3 smooth Gaussian (the prototype's initial condition) to t = 0.2: relative
    L2 error against the FP64 run <= 1e-5, same step count."""
    n = 48
    x = np.linspace(-1, 1, n)
    z, y, xx = np.meshgrid(x, x, x, indexing="ij")
    u0 = np.exp(-(xx ** 2 + y ** 2 + z ** 2) / 0.1)
    h = 2.0 / (n - 1)
    cfg = Weno7Config(n, n, n, h, h, h)
    a64 = _t(u0.ravel(), cuda)
    a32 = _t(u0.ravel().astype(np.float32), cuda)
    t64, it64 = weno7_run(cfg, a64, 0.2, 0.4)
    t32, it32 = weno7_run(cfg, a32, 0.2, 0.4)
    assert it32 == it64
    ref = a64.cpu().numpy()
    rel = np.linalg.norm(a32.cpu().numpy().astype(np.float64) - ref) / np.linalg.norm(ref)
    assert rel <= 1e-5, rel
