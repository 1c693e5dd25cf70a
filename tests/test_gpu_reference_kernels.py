"""The library's FP64 paths against the reference's own CUDA kernels on the same GPU.

The reference's kernels are compiled from its sources (oracle/ref_build.py; -fmad=false, so every
operation is rounded as written, like the oracle) and driven by oracle/ref_gpu.py with the
reference's launch geometry and host loop. The library's FP64 results must equal them bit for
bit: 3D heat O4 + SSP-RK3 (the baseline code), the reference's O2 kernel with forward Euler, 2D
heat O4 + SSP-RK3, and the full Burgers loop (local LF WENO5-Z, viscous term with its doubled
slabs, frozen layers, fixed dt). The cubins are built where the reference sources are; without
them these tests skip.
"""
import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig, HeatConfig, burgers_run, heat_run

pytestmark = pytest.mark.gpu

ref_gpu = pytest.importorskip("oracle.ref_gpu")


def _need(name):
    if not ref_gpu.available(name):
        pytest.skip(f"reference cubin {name} not built (needs the reference sources at build time)")


@pytest.fixture(scope="module")
def mods(cuda):
    out = {}
    yield out
    for m in out.values():
        m.close()


def _mod(mods, name):
    _need(name)
    key = name + "_nofma"
    if key not in mods:
        mods[key] = ref_gpu.RefModule(name, nofma=True)
    return mods[key]


def _rand(n, seed, cuda):
    import torch
    rng = np.random.default_rng(seed)
    return torch.from_numpy(rng.random(n)).to(cuda)


@pytest.mark.parametrize("shape,iters", [((41, 39, 37), 6), ((64, 64, 64), 3)])
def test_heat3d_o4_rk3_equals_reference_kernels(cuda, native, mods, shape, iters):
    import torch
    mod = _mod(mods, "heat3d")
    cfg = HeatConfig.reference_3d(1.0, 10, 10, 10, *shape)
    u = _rand(cfg.numel, 1, cuda)
    ref = u.clone()
    ref_gpu.heat3d_run(mod, ref, *shape, cfg.kx, cfg.ky, cfg.kz, cfg.dt, iters)
    heat_run(cfg, u, iters)
    torch.cuda.synchronize()
    assert torch.equal(u, ref)


def test_heat3d_o2_euler_equals_reference_o2_kernel(cuda, native, mods):
    """The reference's (unused) O2 kernel takes 12*k_a as its coefficient and its RK keeps two
    frozen layers: the same scheme is order 2, frozen 2, coefficients 12 k_a."""
    import torch
    mod = _mod(mods, "heat3d")
    nx, ny, nz = 48, 40, 36
    base = HeatConfig.reference_3d(1.0, 10, 10, 10, nx, ny, nz)
    cfg = HeatConfig(3, nx, ny, nz, 2, 2, False, 12 * base.kx, 12 * base.ky, 12 * base.kz, base.dt, N.ADV_EULER)
    u = _rand(cfg.numel, 2, cuda)
    ref = u.clone()
    ref_gpu.heat3d_run(mod, ref, nx, ny, nz, base.kx, base.ky, base.kz, base.dt, 9, scheme="o2-euler")
    heat_run(cfg, u, 9)
    torch.cuda.synchronize()
    assert torch.equal(u, ref)


def test_heat2d_o4_rk3_equals_reference_kernels(cuda, native, mods):
    import torch
    mod = _mod(mods, "heat2d")
    nx, ny = 256, 128
    cfg = HeatConfig.reference_2d(1.0, 10, 10, nx, ny)
    u = _rand(cfg.numel, 3, cuda)
    ref = u.clone()
    ref_gpu.heat2d_run(mod, ref, nx, ny, cfg.kx, cfg.ky, cfg.dt, 11)
    heat_run(cfg, u, 11)
    torch.cuda.synchronize()
    assert torch.equal(u, ref)


@pytest.mark.parametrize("n,tEnd", [(48, 0.06), (64, 0.05)])
def test_burgers3d_loop_equals_reference_kernels(cuda, native, mods, n, tEnd):
    import torch
    mod = _mod(mods, "burgers3d")
    cfg = BurgersConfig.reference(2.0, 2.0, 2.0, n, n, n, bug_b2=True)
    u0 = np.empty(cfg.numel)
    N.check(N.load().adv_ic_burgers_ref(n, n, n, cfg.dx, cfg.dy, cfg.dz,
                                        u0.ctypes.data_as(N.C.POINTER(N.C.c_double))), "ic")
    u = torch.from_numpy(u0).to(cuda)
    ref = u.clone()
    t_ref, it_ref = ref_gpu.burgers3d_run(mod, ref, n, 2.0, tEnd, 0.3)
    t, it = burgers_run(cfg, u, tEnd, 0.3, dt_rule=N.ADV_DT_FIXED)
    torch.cuda.synchronize()
    assert (t, it) == (t_ref, it_ref)
    assert torch.equal(u, ref)


@pytest.mark.parametrize("shape,iters", [((41, 37, 35), 4), ((64, 64, 48), 3)])
def test_heat3d_blocking_equals_reference_kernels(cuda, oracle, mods, shape, iters):
    """SingleGPU/Diffusion3d_Blocking's own kernels (its blocked Laplacian over 16-plane z blocks,
    its launch geometry) against the compatibility library's Call_Lu3d / Call_RK3d and the
    oracle's restatement: bit for bit. nz avoids the sizes where the reference's last z block
    would read past the array (nz mod 16 of 1 or 2)."""
    import ctypes as C
    import torch
    mod = _mod(mods, "heat3d_blocking")
    nx, ny, nz = shape
    cfg = HeatConfig.reference_3d(1.0, 10, 10, 10, *shape)
    u = _rand(cfg.numel, 3, cuda)
    u0 = u.cpu().numpy()
    ref = u.clone()
    ref_gpu.heat3d_blocking_run(mod, ref, nx, ny, nz, cfg.kx, cfg.ky, cfg.kz, cfg.dt, iters)
    lib = C.CDLL(str(N.LIBDIR / "libadvdiff_compat_heat3d_blocking.so"))

    class Dim3(C.Structure):
        _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]
    uo, Lu = torch.empty_like(u), torch.zeros_like(u)
    lib.CopyToConstantMemory(C.c_double(cfg.kx), C.c_double(cfg.ky), C.c_double(cfg.kz))
    dd = [C.c_uint(nx), C.c_uint(nx), C.c_uint(ny), C.c_uint(nz)]
    pu, puo, pL = (C.c_void_p(x.data_ptr()) for x in (u, uo, Lu))
    for _ in range(iters):
        uo.copy_(u)
        for st in (1, 2, 3):
            lib.Call_Lu3d(Dim3(1, 1, 1), Dim3(32, 4, 1), None, *dd, pu, pL)
            lib.Call_RK3d(Dim3(1, 1, 1), Dim3(32, 4, 4), None, C.c_uint(st), *dd, C.c_double(cfg.dt), pu, puo, pL)
    torch.cuda.synchronize()
    assert lib.adv_compat_last_status() == 0
    assert torch.equal(u, ref)
    want = oracle.heat_blocking_run(nx, ny, nz, cfg.kx, cfg.ky, cfg.kz, cfg.dt, iters, u0)
    np.testing.assert_array_equal(ref.cpu().numpy(), want)
