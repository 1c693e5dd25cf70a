"""The reference's own extern "C" names (compatibility libraries) driven the way the reference's
main.cpp drives them, against the oracle's restatement of the same loop: bit-exact in FP64."""
import ctypes as C

import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig, HeatConfig

pytestmark = pytest.mark.gpu


class Dim3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


def _shim(name):
    lib = C.CDLL(str(N.LIBDIR / name))
    return lib


def _t(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def _padded(a, nx, ny, nz, pitch, cuda):
    import torch
    h = np.zeros((nz, ny, pitch))
    h[:, :, :nx] = a.reshape(nz, ny, nx)
    return torch.from_numpy(h.ravel()).to(cuda)


@pytest.mark.parametrize("pitched", [False, True])
def test_compat_heat3d_loop(cuda, oracle, pitched):
    """main.cpp:106-122: uo <- u; (Call_Lu3d; Call_RK3d(step)) for step = 1..3, five iterations."""
    import torch
    nx, ny, nz, iters = 33, 29, 31, 5
    lib = _shim("libadvdiff_compat_heat3d_pitched.so" if pitched else "libadvdiff_compat_heat3d.so")
    cfg = HeatConfig.reference_3d(1.0, 10, 10, 10, nx, ny, nz)
    dx, dy, dz = 10 / (nx - 1), 10 / (ny - 1), 10 / (nz - 1)
    u0 = oracle.ic_heat_ref(3, nx, ny, nz, dx, dy, dz)
    want = oracle.heat_run(cfg, u0, iters, 1)
    pitch = 40 if pitched else nx
    u = _padded(u0, nx, ny, nz, pitch, cuda)
    uo = torch.empty_like(u)
    Lu = torch.zeros_like(u)
    lib.CopyToConstantMemory(C.c_double(cfg.kx), C.c_double(cfg.ky), C.c_double(cfg.kz))
    g, b = Dim3(1, 1, 1), Dim3(32, 4, 4)
    for _ in range(iters):
        uo.copy_(u)
        for step in (1, 2, 3):
            if pitched:
                lib.Call_Lu3d(g, b, None, C.c_uint(pitch), C.c_uint(nx), C.c_uint(ny), C.c_uint(nz),
                              C.c_void_p(u.data_ptr()), C.c_void_p(Lu.data_ptr()))
                lib.Call_RK3d(g, b, None, C.c_uint(step), C.c_uint(pitch), C.c_uint(nx), C.c_uint(ny), C.c_uint(nz),
                              C.c_double(cfg.dt), C.c_void_p(u.data_ptr()), C.c_void_p(uo.data_ptr()),
                              C.c_void_p(Lu.data_ptr()))
            else:
                lib.Call_Lu3d(g, b, None, C.c_uint(nx), C.c_uint(ny), C.c_uint(nz), C.c_void_p(u.data_ptr()),
                              C.c_void_p(Lu.data_ptr()))
                lib.Call_RK3d(g, b, None, C.c_uint(step), C.c_uint(nx), C.c_uint(ny), C.c_uint(nz), C.c_double(cfg.dt),
                              C.c_void_p(u.data_ptr()), C.c_void_p(uo.data_ptr()), C.c_void_p(Lu.data_ptr()))
    torch.cuda.synchronize()
    assert lib.adv_compat_last_status() == 0
    got = u.cpu().numpy().reshape(nz, ny, pitch)[:, :, :nx].ravel()
    np.testing.assert_array_equal(got, want)


def test_compat_heat2d_loop(cuda, oracle):
    """SingleGPU/Diffusion2d/main.cpp:106-125 (Lu memset per step, three frozen layers)."""
    import torch
    nx, ny, iters = 61, 47, 7
    lib = _shim("libadvdiff_compat_heat2d.so")
    cfg = HeatConfig.reference_2d(1.0, 10, 10, nx, ny)
    u0 = oracle.ic_heat_ref(2, nx, ny, 1, 10 / (nx - 1), 10 / (ny - 1), 0.0)
    want = oracle.heat_run(cfg, u0, iters, 1)
    u = _t(u0, cuda)
    uo = torch.empty_like(u)
    Lu = torch.zeros_like(u)
    lib.CopyToConstantMemory(C.c_double(cfg.kx), C.c_double(cfg.ky))
    g, b = Dim3(4, 3, 1), Dim3(16, 16, 1)
    for _ in range(iters):
        uo.copy_(u)
        Lu.zero_()
        for step in (1, 2, 3):
            lib.Call_Lu2d(g, b, None, C.c_uint(nx), C.c_uint(ny), C.c_void_p(u.data_ptr()), C.c_void_p(Lu.data_ptr()))
            lib.Call_RK2d(g, b, None, C.c_uint(step), C.c_uint(nx), C.c_uint(ny), C.c_double(cfg.dt),
                          C.c_void_p(u.data_ptr()), C.c_void_p(uo.data_ptr()), C.c_void_p(Lu.data_ptr()))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(u.cpu().numpy(), want)


@pytest.mark.parametrize("pitched", [False, True])
def test_compat_burgers_loop(cuda, oracle, pitched):
    """SingleGPU/Burgers3d_WENO5/main.cpp:127-150 with the reference's fixed dt, bug B2 kept."""
    import torch
    nx = ny = nz = 36
    tEnd, cfl, Cv = 0.01, 0.3, 1e-5
    lib = _shim("libadvdiff_compat_burgers3d_pitched.so" if pitched else "libadvdiff_compat_burgers3d.so")
    cfg = BurgersConfig.reference(2.0, 2.0, 2.0, nx, ny, nz, C=Cv, bug_b2=True)
    u0 = oracle.ic_burgers_ref(nx, ny, nz, cfg.dx, cfg.dy, cfg.dz)
    want, t_w, it_w = oracle.burgers_run(cfg, u0, tEnd, cfl, 0, C_visc=Cv)
    pitch = 40 if pitched else nx
    u = _padded(u0, nx, ny, nz, pitch, cuda)
    uo = torch.empty_like(u)
    Lu = torch.zeros_like(u)
    lib.CopyToConstantMemory(*[C.c_double(Cv / (12 * h * h)) for h in (cfg.dx, cfg.dy, cfg.dz)])
    g, b = Dim3(1, 1, 1), Dim3(8, 8, 8)
    P = [C.c_uint(pitch)] if pitched else []
    dims = [C.c_uint(nx), C.c_uint(ny), C.c_uint(nz)]
    pu, puo, pL = (C.c_void_p(x.data_ptr()) for x in (u, uo, Lu))
    t, it = 0.0, 0
    while t < tEnd:
        dt1 = cfl * cfg.dx / 1.0
        dt2 = 1.0 / (2 * Cv * (1 / cfg.dx ** 2 + 1 / cfg.dy ** 2 + 1 / cfg.dz ** 2)) * 0.9
        dt = min(dt1, dt2)
        if t + dt > tEnd:
            dt = tEnd - t
        t += dt
        it += 1
        uo.copy_(u)
        for step in (1, 2, 3):
            lib.Call_Adv_x(g, b, None, *P, *dims, C.c_double(cfg.dx), pu, pL)
            lib.Call_Adv_y(g, b, None, *P, *dims, C.c_double(cfg.dy), pu, pL)
            lib.Call_Adv_z(g, b, None, *P, *dims, C.c_double(cfg.dz), pu, pL)
            lib.Call_Diff_(g, b, None, *P, *dims, pu, pL)
            lib.Call_sspRK(g, b, None, *P, *dims, C.c_uint(step), C.c_double(dt), pu, puo, pL)
    torch.cuda.synchronize()
    assert it == it_w and t == t_w
    got = u.cpu().numpy().reshape(nz, ny, pitch)[:, :, :nx].ravel()
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("dims,pitch", [((33, 29, 31), 40), ((41, 37, 35), 41)])
def test_compat_heat3d_blocking_loop(cuda, oracle, dims, pitch):
    """SingleGPU/Diffusion3d_Blocking/main.cpp:101-123 through its own names (pitched signatures,
    Lu zeroed once): the Laplacian on i, j in [3, n-4], k in [3, nz-3], the stage update on
    [2, n-3]; equal to the oracle's restatement bit for bit."""
    import torch
    nx, ny, nz = dims
    iters = 5
    lib = _shim("libadvdiff_compat_heat3d_blocking.so")
    cfg = HeatConfig.reference_3d(1.0, 10, 10, 10, nx, ny, nz)
    u0 = oracle.ic_heat_ref(3, nx, ny, nz, 10 / (nx - 1), 10 / (ny - 1), 10 / (nz - 1))
    want = oracle.heat_blocking_run(nx, ny, nz, cfg.kx, cfg.ky, cfg.kz, cfg.dt, iters, u0)
    u = _padded(u0, nx, ny, nz, pitch, cuda)
    uo = torch.empty_like(u)
    Lu = torch.zeros_like(u)
    lib.CopyToConstantMemory(C.c_double(cfg.kx), C.c_double(cfg.ky), C.c_double(cfg.kz))
    g2, b2, g3, b3 = Dim3(1, 1, 1), Dim3(32, 4, 1), Dim3(1, 1, 1), Dim3(32, 4, 4)
    dd = [C.c_uint(pitch), C.c_uint(nx), C.c_uint(ny), C.c_uint(nz)]
    pu, puo, pL = (C.c_void_p(x.data_ptr()) for x in (u, uo, Lu))
    for _ in range(iters):
        uo.copy_(u)
        for step in (1, 2, 3):
            lib.Call_Lu3d(g2, b2, None, *dd, pu, pL)
            lib.Call_RK3d(g3, b3, None, C.c_uint(step), *dd, C.c_double(cfg.dt), pu, puo, pL)
    torch.cuda.synchronize()
    assert lib.adv_compat_last_status() == 0
    got = u.cpu().numpy().reshape(nz, ny, pitch)[:, :, :nx].ravel()
    np.testing.assert_array_equal(got, want)
    # the blocked program's update differs from the baseline program's (z plane nz-3 takes the
    # Laplacian, the outer update ring does not)
    assert not np.array_equal(want, oracle.heat_run(cfg, u0, iters, 1))


def test_compat_burgers_sharedmem_loop(cuda, oracle):
    """SingleGPU/Burgers3d_WENO5_SharedMem/main.cpp:136-162 through its own names: the
    shared-memory sweeps (every node, zero beyond the grid, reciprocal weight normalisation),
    then the baseline's viscous term and stage update; equal to the oracle bit for bit."""
    import torch
    nx = ny = nz = 36
    pitch = 40
    tEnd, cfl, Cv = 0.01, 0.3, 1e-5
    lib = _shim("libadvdiff_compat_burgers3d_sharedmem.so")
    cfg = BurgersConfig.reference(2.0, 2.0, 2.0, nx, ny, nz, C=Cv, bug_b2=True)
    u0 = oracle.ic_burgers_ref(nx, ny, nz, cfg.dx, cfg.dy, cfg.dz)
    want, t_w, it_w = oracle.burgers_run(cfg, u0, tEnd, cfl, 0, C_visc=Cv, recip=True)
    base, _, _ = oracle.burgers_run(cfg, u0, tEnd, cfl, 0, C_visc=Cv)
    assert not np.array_equal(want, base)  # the normalisations round differently
    u = _padded(u0, nx, ny, nz, pitch, cuda)
    uo = torch.empty_like(u)
    Lu = torch.zeros_like(u)
    lib.CopyToConstantMemory(*[C.c_double(Cv / (12 * h * h)) for h in (cfg.dx, cfg.dy, cfg.dz)])
    g, b = Dim3(1, 1, 1), Dim3(8, 8, 8)
    P = [C.c_uint(pitch), C.c_uint(nx), C.c_uint(ny), C.c_uint(nz)]
    pu, puo, pL = (C.c_void_p(x.data_ptr()) for x in (u, uo, Lu))
    t, it = 0.0, 0
    while t < tEnd:
        dt = min(cfl * cfg.dx / 1.0, 1.0 / (2 * Cv * (1 / cfg.dx ** 2 + 1 / cfg.dy ** 2 + 1 / cfg.dz ** 2)) * 0.9)
        if t + dt > tEnd:
            dt = tEnd - t
        t += dt
        it += 1
        uo.copy_(u)
        for step in (1, 2, 3):
            lib.Call_Adv_x(g, b, None, *P, C.c_double(cfg.dx), pu, pL)
            lib.Call_Adv_y(g, b, None, *P, C.c_double(cfg.dy), pu, pL)
            lib.Call_Adv_z(g, b, None, *P, C.c_double(cfg.dz), pu, pL)
            lib.Call_Diff_(g, b, None, *P, pu, pL)
            lib.Call_sspRK(g, b, None, *P, C.c_uint(step), C.c_double(dt), pu, puo, pL)
    torch.cuda.synchronize()
    assert lib.adv_compat_last_status() == 0
    assert it == it_w and t == t_w
    got = u.cpu().numpy().reshape(nz, ny, pitch)[:, :, :nx].ravel()
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("shape", [(13, 11, 9), (40, 7, 6), (6, 6, 6), (130, 5, 4)])
@pytest.mark.parametrize("weno", [N.ADV_WENO5_Z, N.ADV_WENO5_JS], ids=["z", "js"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_ref_sweep_all_equals_oracle(cuda, native, oracle, shape, weno, dtype):
    """adv_ref_burgers_sweep_all on every node of every line, each axis (x assigns, y and z
    subtract from what is there), lines shorter and longer than the reference's 128-node tile."""
    import torch
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * 7 + ny + nz)
    u = (rng.standard_normal((nz, ny, nx)) * 0.7).astype(dtype)
    Lu0 = rng.standard_normal((nz, ny, nx)).astype(dtype)
    du = _t(u.ravel(), cuda)
    for axis, h in ((0, 0.05), (1, 0.07), (2, 0.11)):
        want = oracle.burgers_sweep_all(axis, weno == N.ADV_WENO5_Z, u, h, Lu0)
        dL = _t(Lu0.ravel(), cuda)
        assert native.adv_ref_burgers_sweep_all(N.ADV_F64 if dtype == np.float64 else N.ADV_F32, axis, weno, nx, nx,
                                                ny, nz, h, C.c_void_p(du.data_ptr()), C.c_void_p(dL.data_ptr()),
                                                None) == N.ADV_OK
        torch.cuda.synchronize()
        np.testing.assert_array_equal(dL.cpu().numpy().reshape(nz, ny, nx), want)
