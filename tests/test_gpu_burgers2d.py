"""2D Burgers: an nx x ny x 1 problem of the fused Burgers stage and loop. The z faces of every
column are equal, so their difference is exactly zero and the 2D update is bit for bit the 3D
update of a z-independent field. FP64 is bit-exact against the oracle; a 2D periodic run equals
every plane of the same field extruded in z; FP32 is held to a stated tolerance."""
import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig, burgers_run, burgers_stage

pytestmark = pytest.mark.gpu


def _t(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def _cfg(kind, nx, ny, weno=N.ADV_WENO5_Z):
    if kind.startswith("periodic"):
        return BurgersConfig(nx, ny, 1, 2.0 / nx, 2.0 / ny, 2.0 / nx, weno,
                             N.ADV_LF_GLOBAL if kind.endswith("global") else N.ADV_LF_LOCAL, N.ADV_BC_PERIODIC)
    c = BurgersConfig.reference_2d(2.0, 2.0, nx, ny, C=1e-2 if "visc" in kind else 0.0)
    c.weno = weno
    return c


def _field(nx, ny, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 2, nx, endpoint=False)[None, :]
    y = np.linspace(0, 2, ny, endpoint=False)[:, None]
    u = 0.5 + 0.4 * np.sin(np.pi * x + 1) * np.cos(np.pi * y)
    return (u + 0.05 * rng.standard_normal(u.shape)).ravel()


CASES = [(k, s, w) for s in [(64, 48), (37, 29), (130, 17)] for w in (N.ADV_WENO5_Z, N.ADV_WENO5_JS)
         for k in ("periodic-global", "periodic-local", "frozen", "frozen-visc")]


@pytest.mark.parametrize("kind,size,weno", CASES)
@pytest.mark.parametrize("stage", [1, 3])
def test_burgers2d_stage_fp64_bitwise(cuda, oracle, kind, size, weno, stage):
    cfg = _cfg(kind, *size, weno)
    uin = _field(*size, stage)
    un = uin if stage == 1 else _field(*size, 50 + stage)
    want = oracle.burgers_stage(cfg, stage, uin, un, 1e-3)
    a = _t(uin, cuda)
    b = a if stage == 1 else _t(un, cuda)
    out = a.new_full(a.shape, np.nan)
    burgers_stage(cfg, stage, a, b, out, 1e-3, float(np.abs(uin).max()))
    np.testing.assert_array_equal(out.cpu().numpy(), want)


@pytest.mark.parametrize("kind", ["periodic-global", "frozen"])
def test_burgers2d_stage_fp32(cuda, oracle, kind):
    """FP32 stage vs the FP32 oracle: max |diff| <= 4e-7 * max|u|."""
    cfg = _cfg(kind, 96, 80)
    uin = _field(96, 80, 7).astype(np.float32)
    un = _field(96, 80, 8).astype(np.float32)
    want = oracle.burgers_stage(cfg, 2, uin, un, 2e-3)
    a, b = _t(uin, cuda), _t(un, cuda)
    out = a.new_full(a.shape, np.nan)
    burgers_stage(cfg, 2, a, b, out, 2e-3, float(np.abs(uin).max()))
    got = out.cpu().numpy()
    assert np.isfinite(got).all()
    assert np.abs(got - want).max() <= 4e-7 * np.abs(want).max()


def test_burgers2d_reference_scheme_run_fp64_bitwise(cuda, oracle, native):
    """The reference's 2D scheme (WENO5-JS, local LF, inviscid, dt = CFL dx, its centred Gaussian
    IC) to t = 0.2 at 101 x 81."""
    nx, ny = 101, 81
    cfg = BurgersConfig.reference_2d(2.0, 2.0, nx, ny)
    u0 = np.empty(nx * ny)
    N.check(native.adv_ic_burgers_ref2d(nx, ny, cfg.dx, cfg.dy, u0.ctypes.data_as(N.C.POINTER(N.C.c_double))), "ic")
    want, t_w, it_w = oracle.burgers_run(cfg, u0, 0.2, 0.3, 0)
    u = _t(u0, cuda)
    t, it = burgers_run(cfg, u, 0.2, 0.3, N.ADV_DT_FIXED)
    assert it == it_w and t == t_w
    np.testing.assert_array_equal(u.cpu().numpy(), want)


def test_burgers2d_viscous_run_fp64_bitwise(cuda, oracle):
    """Viscous frozen 2D run (fixed dt from both the CFL and the 2D diffusion bound)."""
    cfg = _cfg("frozen-visc", 72, 56)
    u0 = _field(72, 56, 11)
    want, t_w, it_w = oracle.burgers_run(cfg, u0, 0.05, 0.3, 0, C_visc=cfg.C)
    u = _t(u0, cuda)
    t, it = burgers_run(cfg, u, 0.05, 0.3, N.ADV_DT_FIXED)
    assert it == it_w and t == t_w
    np.testing.assert_array_equal(u.cpu().numpy(), want)


@pytest.mark.parametrize("weno", [N.ADV_WENO5_Z, N.ADV_WENO5_JS])
def test_burgers2d_periodic_run_equals_extruded_3d(cuda, oracle, weno):
    """dt = CFL dx / max|u|, global LF: a 2D periodic run equals the oracle, and every plane of the
    3D run of the same field extruded over 8 planes, bit for bit."""
    import torch
    nx, ny, nz = 64, 40, 8
    c2 = _cfg("periodic-global", nx, ny, weno)
    c3 = BurgersConfig(nx, ny, nz, c2.dx, c2.dy, c2.dx, weno, N.ADV_LF_GLOBAL, N.ADV_BC_PERIODIC)
    u0 = _field(nx, ny, 5)
    want, t_w, it_w = oracle.burgers_run(c2, u0, 0.4, 0.4, 1)
    u2 = _t(u0, cuda)
    t2, it2 = burgers_run(c2, u2, 0.4, 0.4, N.ADV_DT_MAXU)
    assert (t2, it2) == (t_w, it_w)
    np.testing.assert_array_equal(u2.cpu().numpy(), want)
    u3 = _t(np.tile(u0, nz), cuda)
    t3, it3 = burgers_run(c3, u3, 0.4, 0.4, N.ADV_DT_MAXU)
    assert (t3, it3) == (t2, it2)
    assert torch.equal(u3.view(nz, -1), u2.view(1, -1).expand(nz, -1))


def test_burgers2d_fp32_run_vs_fp64_oracle(cuda, oracle):
    """FP32 state to t = 0.5 (past shock formation) within 1e-5 relative L2 of the FP64 oracle."""
    cfg = _cfg("periodic-global", 128, 96)
    u0 = _field(128, 96, 9)
    want, _, it_w = oracle.burgers_run(cfg, u0, 0.5, 0.4, 1)
    u = _t(u0.astype(np.float32), cuda)
    _, it = burgers_run(cfg, u, 0.5, 0.4, N.ADV_DT_MAXU)
    assert abs(it - it_w) <= 1
    got = u.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-5
