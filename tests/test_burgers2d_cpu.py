"""2D Burgers (nz = 1) on the CPU: the oracle's 2D scheme against the 3D scheme of a z-extruded
field, the reference's 2D initial condition, and the descriptor checks of the library."""
import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig


def _field(nx, ny, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 2, nx, endpoint=False)[None, :]
    y = np.linspace(0, 2, ny, endpoint=False)[:, None]
    return (0.5 + 0.4 * np.sin(np.pi * x) * np.cos(np.pi * y + 1) + 0.05 * rng.standard_normal((ny, nx))).ravel()


@pytest.mark.parametrize("weno", [N.ADV_WENO5_Z, N.ADV_WENO5_JS])
def test_oracle_2d_periodic_run_equals_extruded_3d(oracle, weno):
    nx, ny, nz = 24, 18, 6
    h = 2.0 / nx
    c2 = BurgersConfig(nx, ny, 1, h, 2.0 / ny, h, weno, N.ADV_LF_LOCAL, N.ADV_BC_PERIODIC)
    c3 = BurgersConfig(nx, ny, nz, h, 2.0 / ny, h, weno, N.ADV_LF_LOCAL, N.ADV_BC_PERIODIC)
    u0 = _field(nx, ny, 1)
    u2, t2, it2 = oracle.burgers_run(c2, u0, 0.3, 0.4, 1)
    u3, t3, it3 = oracle.burgers_run(c3, np.tile(u0, nz), 0.3, 0.4, 1)
    assert (t2, it2) == (t3, it3) and it2 > 5
    np.testing.assert_array_equal(u3.reshape(nz, -1), np.broadcast_to(u2, (nz, u2.size)))


def test_oracle_2d_frozen_layers_stay(oracle):
    cfg = BurgersConfig.reference_2d(2.0, 2.0, 30, 20, C=1e-3)
    u0 = _field(30, 20, 2)
    out = oracle.burgers_stage(cfg, 1, u0, u0, 1e-3).reshape(20, 30)
    a = u0.reshape(20, 30)
    for sl in (np.s_[:3, :], np.s_[-3:, :], np.s_[:, :3], np.s_[:, -3:]):
        np.testing.assert_array_equal(out[sl], a[sl])
    assert not np.array_equal(out[3:-3, 3:-3], a[3:-3, 3:-3])


def test_ic_burgers_ref2d(native):
    nx, ny, dx, dy = 21, 17, 0.1, 0.125
    u = np.empty(nx * ny)
    assert native.adv_ic_burgers_ref2d(nx, ny, dx, dy, u.ctypes.data_as(N.C.POINTER(N.C.c_double))) == N.ADV_OK
    i = np.arange(nx)[None, :]
    j = np.arange(ny)[:, None]
    x, y = (0.5 * (nx - 1) - i) * dx, (0.5 * (ny - 1) - j) * dy
    want = np.exp(-(x * x + y * y) / 0.1)
    want[0, :] = want[-1, :] = 0
    want[:, 0] = want[:, -1] = 0
    np.testing.assert_allclose(u.reshape(ny, nx), want, rtol=1e-15, atol=0)
    assert u.reshape(ny, nx)[ny // 2, nx // 2] == 1.0


def _ws(native, d):
    nb = N.C.c_size_t(0)
    return native.adv_burgers_workspace_bytes(N.C.byref(d), N.C.byref(nb))


def test_2d_descriptor_checks(native):
    d = BurgersConfig.reference_2d(2.0, 2.0, 32, 32, C=1e-3).desc(N.ADV_F64)
    assert d.kz == 0.0 and _ws(native, d) == N.ADV_OK
    d.kz = 1.0  # a 2D grid has no z term
    assert _ws(native, d) == N.ADV_ERR_INVALID_ARG
    p = BurgersConfig(8, 6, 1, 0.25, 0.25, 0.25, N.ADV_WENO5_Z, N.ADV_LF_GLOBAL, N.ADV_BC_PERIODIC).desc(N.ADV_F32)
    assert _ws(native, p) == N.ADV_OK  # periodic 2D needs 6 cells in x and y only
    p.ny = 5
    assert _ws(native, p) == N.ADV_ERR_INVALID_ARG


def test_2d_adjoint_rejected(native):
    d = BurgersConfig(16, 16, 1, 0.125, 0.125, 0.125, N.ADV_WENO5_Z, N.ADV_LF_LOCAL, N.ADV_BC_PERIODIC).desc(N.ADV_F64)
    nb = N.C.c_size_t(0)
    assert native.adv_burgers_checkpoint_bytes(N.C.byref(d), 10, 5, N.C.byref(nb), N.C.byref(nb)) == N.ADV_ERR_UNSUPPORTED
