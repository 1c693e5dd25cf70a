"""Fused heat stage on the GPU against the oracle: bit-exact (FP32 and FP64), both load paths
(TMA for 16-byte-aligned rows, cp.async otherwise), every stage, 2D and 3D, O2 and O4."""
import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import HeatConfig, heat_run, heat_stage

pytestmark = pytest.mark.gpu


def _cfg(ndim, order, nx, ny, nz, frozen, zero, time=N.ADV_SSPRK3):
    rng = np.random.default_rng(nx * 131 + ny * 7 + nz)
    k = rng.uniform(0.01, 0.05, 3)
    return HeatConfig(ndim, nx, ny, nz if ndim == 3 else 1, order, frozen, zero, *k, 0.7, time)


def _t(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


SIZES3 = [(64, 40, 24), (37, 29, 23), (5, 6, 7), (130, 9, 17), (256, 12, 5), (160, 50, 17), (192, 33, 40), (132, 70, 9)]
SIZES2 = [(64, 40), (37, 29), (6, 5), (300, 17)]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", [2, 4])
@pytest.mark.parametrize("size", SIZES3)
@pytest.mark.parametrize("stage", [1, 2, 3])
def test_heat3d_stage_bitwise(cuda, oracle, dtype, order, size, stage):
    nx, ny, nz = size
    R = order // 2
    for frozen, zero in ((R, True), (R + 1, False)):
        if min(size) < 2 * frozen + 1:
            continue
        cfg = _cfg(3, order, nx, ny, nz, frozen, zero)
        rng = np.random.default_rng(stage)
        uin = rng.standard_normal(nx * ny * nz).astype(dtype)
        un = uin if stage == 1 else rng.standard_normal(nx * ny * nz).astype(dtype)
        want = oracle.heat_stage(cfg, stage, uin, un)
        a, b = _t(uin, cuda), _t(un, cuda) if stage != 1 else None
        b = a if stage == 1 else b
        out = a.new_full(a.shape, np.nan)
        heat_stage(cfg, stage, a, b, out)
        np.testing.assert_array_equal(out.cpu().numpy(), want)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("order", [2, 4])
@pytest.mark.parametrize("size", SIZES2)
@pytest.mark.parametrize("stage", [1, 3])
def test_heat2d_stage_bitwise(cuda, oracle, dtype, order, size, stage):
    nx, ny = size
    frozen = 3 if order == 4 else 1
    if min(size) < 2 * frozen + 1:
        pytest.skip("grid smaller than the frozen layers")
    cfg = _cfg(2, order, nx, ny, 1, frozen, order == 2)
    rng = np.random.default_rng(11)
    uin = rng.standard_normal(nx * ny).astype(dtype)
    un = uin if stage == 1 else rng.standard_normal(nx * ny).astype(dtype)
    want = oracle.heat_stage(cfg, stage, uin, un)
    a = _t(uin, cuda)
    b = a if stage == 1 else _t(un, cuda)
    out = a.new_full(a.shape, np.nan)
    heat_stage(cfg, stage, a, b, out)
    np.testing.assert_array_equal(out.cpu().numpy(), want)


def test_heat_stage_stage3_in_place_into_un(cuda, oracle):
    cfg = _cfg(3, 4, 40, 24, 20, 2, False)
    rng = np.random.default_rng(5)
    uin = rng.standard_normal(40 * 24 * 20)
    un = rng.standard_normal(40 * 24 * 20)
    want = oracle.heat_stage(cfg, 3, uin, un)
    a, b = _t(uin, cuda), _t(un, cuda)
    heat_stage(cfg, 3, a, b, b)
    np.testing.assert_array_equal(b.cpu().numpy(), want)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("time,nsteps", [(N.ADV_EULER, 1), (N.ADV_EULER, 71), (N.ADV_EULER, 130), (N.ADV_SSPRK3, 1),
                                         (N.ADV_SSPRK3, 37)])
def test_heat_run_bitwise(cuda, oracle, dtype, time, nsteps):
    """adv_heat_run (CUDA-graph replay of captured chunks + remainder) equals the oracle loop."""
    if time == N.ADV_EULER:
        cfg = HeatConfig.dirichlet_o2(3, 36)
        u0 = oracle.ic_heat3d_blobs(36, 36, 36, 2)
    else:
        cfg = HeatConfig.reference_3d(1.0, 10, 10, 10, 33, 31, 29)
        u0 = oracle.ic_heat_ref(3, 33, 31, 29, 10 / 32, 10 / 30, 10 / 28)
    u0 = u0.astype(dtype)
    want = oracle.heat_run(cfg, u0, nsteps, time)
    u = _t(u0, cuda)
    heat_run(cfg, u, nsteps)
    np.testing.assert_array_equal(u.cpu().numpy(), want)


def test_heat2d_config_c1_bitwise(cuda, oracle):
    """2D heat, 512^2 FP32, O2 forward Euler r = 0.2, Dirichlet, bump + N(0,1e-3) noise, 1000 steps."""
    cfg = HeatConfig.dirichlet_o2(2, 512)
    u0 = oracle.ic_heat2d_gauss_noise(512, 512, 1, 1e-3).astype(np.float32)
    want = oracle.heat_run(cfg, u0, 1000, 0)
    u = _t(u0, cuda)
    heat_run(cfg, u, 1000)
    np.testing.assert_array_equal(u.cpu().numpy(), want)


def test_heat3d_config_c2_full_size(cuda, oracle):
    """3D heat at 256^3, O2 Euler r = 1/8, Dirichlet, 8 seeded blobs: FP32 and FP64 bit-exact with the
    oracle over 8 steps; over the full 2000 steps FP32 stays within 1e-5 relative L2 of FP64, obeys
    the maximum principle and keeps the boundary at zero."""
    import torch
    n = 256
    cfg = HeatConfig.dirichlet_o2(3, n)
    u0 = oracle.ic_heat3d_blobs(n, n, n, 2)
    for dt in (np.float32, np.float64):
        want = oracle.heat_run(cfg, u0.astype(dt), 8, 0)
        u = _t(u0.astype(dt), cuda)
        heat_run(cfg, u, 8)
        np.testing.assert_array_equal(u.cpu().numpy(), want)
    u32 = _t(u0.astype(np.float32), cuda)
    u64 = _t(u0, cuda)
    heat_run(cfg, u32, 2000)
    heat_run(cfg, u64, 2000)
    rel = (torch.linalg.vector_norm(u32.double() - u64) / torch.linalg.vector_norm(u64)).item()
    assert rel <= 1e-5, rel
    v = u64.view(n, n, n)
    assert v.max().item() <= float(u0.max()) and v.min().item() >= 0.0
    assert v[0].abs().max().item() == 0.0 and v[:, :, -1].abs().max().item() == 0.0


def test_heat3d_reference_grid_bitwise(cuda, oracle):
    """The reference's own 3D run (201 x 199 x 200, O4 + SSP-RK3, FP64; rows of 201 doubles are not
    16-byte multiples, so this is the cp.async path): bit-exact over 6 steps."""
    cfg = HeatConfig.reference_3d(1.0, 10, 10, 10, 201, 199, 200)
    u0 = oracle.ic_heat_ref(3, 201, 199, 200, 10 / 200, 10 / 198, 10 / 199)
    want = oracle.heat_run(cfg, u0, 6, 1)
    u = _t(u0, cuda)
    heat_run(cfg, u, 6)
    np.testing.assert_array_equal(u.cpu().numpy(), want)


def test_heat_rejects_bad_arguments(cuda):
    import torch
    cfg = HeatConfig.dirichlet_o2(3, 16)
    a = torch.zeros(16 ** 3, device=cuda)
    with pytest.raises(N.AdvError) as e:
        heat_stage(cfg, 1, a, a, a)  # u_in aliases u_out
    assert e.value.status == N.ADV_ERR_INVALID_ARG
    with pytest.raises(N.AdvError):
        heat_stage(cfg, 4, a, a, torch.zeros_like(a))


@pytest.mark.parametrize("order,ndim,time,nsteps", [(2, 3, N.ADV_EULER, 9), (4, 3, N.ADV_SSPRK3, 4), (2, 2, N.ADV_EULER, 7),
                                                    (4, 2, N.ADV_SSPRK3, 3)])
@pytest.mark.parametrize("size", [(64, 40, 24), (37, 29, 23)])
def test_heat_fp64_contracted_form(cuda, oracle, order, ndim, time, nsteps, size):
    """FP64 with contract = 1 (the fused multiply-add pattern): bit-exact against the oracle's
    mirror of that pattern, on both load paths (rows of 16-byte multiples take TMA, odd rows
    cp.async), and within 8 ulps of the magnitude of the state of the reference's rounding."""
    import dataclasses
    nx, ny, nz = size
    R = order // 2
    cfg = _cfg(ndim, order, nx, ny, nz, R + (1 if order == 4 else 0), order == 2, time)
    fma = dataclasses.replace(cfg, contract=True)
    u0 = np.random.default_rng(3).standard_normal(cfg.numel)
    want = oracle.heat_run(fma, u0, nsteps, time)
    u = _t(u0, cuda)
    heat_run(fma, u, nsteps)
    got = u.cpu().numpy()
    np.testing.assert_array_equal(got, want)
    exact = oracle.heat_run(cfg, u0, nsteps, time)
    assert np.abs(got - exact).max() <= 8 * np.finfo(np.float64).eps * np.abs(exact).max()
