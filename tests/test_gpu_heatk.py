"""Heat with a diffusivity field k(x) and its discrete adjoint on the GPU (adv_heatk_*).

One step and one adjoint step equal the oracle bit for bit (FP32 and FP64); the checkpointed
backward run (any checkpoint interval) gives exactly the oracle's gradient computed by storing
every state; the gradient agrees with central differences of the FP64 forward run and the FP32
gradient with the FP64 one."""
import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import HeatKConfig, heatk_adjoint_step, heatk_run, heatk_step

pytestmark = pytest.mark.gpu


def _case(shape, dtype, seed, zero_boundary=True):
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    k = np.exp(0.5 * rng.standard_normal(n))
    c = 0.15 / k.max()
    cfg = HeatKConfig(*shape, c, c * 0.9, c * 1.1, zero_boundary)
    u0 = rng.random(n)
    if zero_boundary:
        u0.reshape(shape[::-1])[[0, -1], :, :] = 0
    target = rng.random(n)
    return cfg, k.astype(dtype), u0.astype(dtype), target.astype(dtype)


def _t(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


@pytest.mark.parametrize("shape", [(37, 29, 33), (40, 29, 33)], ids=["scalar-rows", "vector-rows"])
@pytest.mark.parametrize("zb", [True, False], ids=["zero", "held"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_step_and_adjoint_step_equal_oracle(cuda, native, oracle, dtype, zb, shape):
    import torch
    cfg, k, u, _ = _case(shape, dtype, 1, zb)
    rng = np.random.default_rng(9)
    lam = rng.standard_normal(u.size).astype(dtype)
    g0 = rng.standard_normal(u.size).astype(dtype)
    c = (cfg.cx, cfg.cy, cfg.cz)
    want_u = oracle.heatk_step(shape, zb, c, k, u)
    g_want = g0.copy()
    want_l = oracle.heatk_adjoint(shape, zb, c, k, u, lam, g_want)
    dk, du, dl, dg = _t(k, cuda), _t(u, cuda), _t(lam, cuda), _t(g0, cuda)
    out = torch.empty_like(du)
    lo = torch.empty_like(dl)
    heatk_step(cfg, dk, du, out)
    heatk_adjoint_step(cfg, dk, du, dl, lo, dg)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), want_u)
    assert np.array_equal(lo.cpu().numpy(), want_l)
    assert np.array_equal(dg.cpu().numpy(), g_want)


@pytest.mark.parametrize("interval", [1, 3, 4, 10, 16])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_checkpointed_gradient_equals_oracle(cuda, native, oracle, dtype, interval):
    import torch
    shape = (24, 20, 18)
    steps = 10
    cfg, k, u0, target = _case(shape, dtype, 2)
    c = (cfg.cx, cfg.cy, cfg.cz)
    J, gk, gu = oracle.heatk_loss_and_gradient(shape, True, c, k, u0, target, steps)
    dk = _t(k, cuda).requires_grad_(True)
    du = _t(u0, cuda).requires_grad_(True)
    uT = heatk_run(cfg, dk, du, steps, interval)
    loss = 0.5 * ((uT - _t(target, cuda)) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    assert np.array_equal(dk.grad.cpu().numpy(), gk)
    assert np.array_equal(du.grad.cpu().numpy(), gu)


@pytest.mark.parametrize("shape", [(136, 20, 40), (64, 9, 70), (128, 33, 7)], ids=["two-x-tiles", "z-chunks", "thin"])
@pytest.mark.parametrize("zb", [True, False], ids=["zero", "held"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_checkpointed_gradient_shapes_equal_oracle(cuda, native, oracle, dtype, zb, shape):
    """The checkpointed gradient equals the oracle's bit for bit across several x tiles, several z
    chunks per column, held and zeroed boundaries, and a last segment shorter than the interval."""
    import torch
    steps = 9
    cfg, k, u0, target = _case(shape, dtype, 4, zb)
    c = (cfg.cx, cfg.cy, cfg.cz)
    J, gk, gu = oracle.heatk_loss_and_gradient(shape, zb, c, k, u0, target, steps)
    dk = _t(k, cuda).requires_grad_(True)
    du = _t(u0, cuda).requires_grad_(True)
    uT = heatk_run(cfg, dk, du, steps, 5)
    loss = 0.5 * ((uT - _t(target, cuda)) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    assert np.array_equal(dk.grad.cpu().numpy(), gk)
    assert np.array_equal(du.grad.cpu().numpy(), gu)


def test_gradient_matches_central_differences_fp64(cuda, native):
    import torch
    shape = (32, 32, 32)
    steps = 30
    cfg, k, u0, target = _case(shape, np.float64, 3)
    dk, du, dt_ = _t(k, cuda), _t(u0, cuda), _t(target, cuda)

    def J(kk, uu):
        with torch.no_grad():
            uT = heatk_run(cfg, kk, uu, steps)
            return 0.5 * float(((uT - dt_) ** 2).sum())

    kk = dk.clone().requires_grad_(True)
    uu = du.clone().requires_grad_(True)
    loss = 0.5 * ((heatk_run(cfg, kk, uu, steps) - dt_) ** 2).sum()
    loss.backward()
    rng = np.random.default_rng(5)
    for _ in range(4):
        vk = _t(rng.standard_normal(k.size), cuda)
        vu = _t(rng.standard_normal(k.size), cuda)
        eps = 1e-6
        fd = (J(dk + eps * vk, du + eps * vu) - J(dk - eps * vk, du - eps * vu)) / (2 * eps)
        ad = float((kk.grad * vk).sum() + (uu.grad * vu).sum())
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def test_fp32_gradient_close_to_fp64(cuda, native):
    import torch
    shape = (48, 40, 36)
    steps = 40
    cfg, k, u0, target = _case(shape, np.float64, 4)
    grads = {}
    for dt in (torch.float32, torch.float64):
        kk = _t(k, cuda).to(dt).requires_grad_(True)
        uu = _t(u0, cuda).to(dt).requires_grad_(True)
        loss = 0.5 * ((heatk_run(cfg, kk, uu, steps) - _t(target, cuda).to(dt)) ** 2).sum()
        loss.backward()
        grads[dt] = kk.grad.double()
    g32, g64 = grads[torch.float32], grads[torch.float64]
    rel = (torch.linalg.vector_norm(g32 - g64) / torch.linalg.vector_norm(g64)).item()
    assert rel < 1e-5, rel


def test_backward_rejects_bad_interval(cuda, native):
    d = HeatKConfig(8, 8, 8, 0.1, 0.1, 0.1).desc(N.ADV_F32)
    cb, wb = N.C.c_size_t(0), N.C.c_size_t(0)
    assert native.adv_heatk_checkpoint_bytes(N.C.byref(d), 10, 0, N.C.byref(cb), N.C.byref(wb)) == N.ADV_ERR_INVALID_ARG
    assert native.adv_heatk_checkpoint_bytes(N.C.byref(d), 10, 4, N.C.byref(cb), N.C.byref(wb)) == N.ADV_OK
    one = (8 * 8 * 8 * 4 + 255) // 256 * 256
    assert cb.value == 3 * one and wb.value == 4 * one


@pytest.mark.parametrize("steps,interval", [(10, 4), (12, 4), (7, 7), (9, 1), (1, 3)])
def test_backward_with_and_without_the_kept_interval(cuda, native, oracle, steps, interval):
    """adv_heatk_forward leaves its last interval's states in work; the backward run that takes
    them (ADV_HEATK_LAST_INTERVAL_IN_WORK) and the one that recomputes them (flags 0) give the same
    bits, for last intervals of every length, and the forward's result is the plain run's."""
    import torch
    shape = (24, 20, 18)
    cfg, k, u0, target = _case(shape, np.float32, 2)
    d = cfg.desc(N.ADV_F32)
    cb, wb = N.C.c_size_t(0), N.C.c_size_t(0)
    assert native.adv_heatk_checkpoint_bytes(N.C.byref(d), steps, interval, N.C.byref(cb), N.C.byref(wb)) == N.ADV_OK
    kk = _t(k, cuda)
    res = []
    for flags in (N.ADV_HEATK_LAST_INTERVAL_IN_WORK, 0):
        u = _t(u0, cuda)
        ckpt = torch.empty(cb.value, dtype=torch.uint8, device=cuda)
        work = torch.empty(wb.value, dtype=torch.uint8, device=cuda)
        assert native.adv_heatk_forward(N.C.byref(d), kk.data_ptr(), u.data_ptr(), steps, interval, ckpt.data_ptr(),
                                        work.data_ptr(), None) == N.ADV_OK
        plain = _t(u0, cuda)
        w2 = torch.empty_like(plain)
        assert native.adv_heatk_forward(N.C.byref(d), kk.data_ptr(), plain.data_ptr(), steps, interval, None,
                                        w2.data_ptr(), None) == N.ADV_OK
        assert torch.equal(u, plain)
        lam = u - _t(target, cuda)
        gk = torch.zeros_like(kk)
        assert native.adv_heatk_backward(N.C.byref(d), kk.data_ptr(), steps, interval, ckpt.data_ptr(),
                                         lam.data_ptr(), gk.data_ptr(), work.data_ptr(), flags, None) == N.ADV_OK
        torch.cuda.synchronize()
        res.append((lam.cpu().numpy(), gk.cpu().numpy()))
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])
    assert native.adv_heatk_backward(N.C.byref(d), kk.data_ptr(), steps, interval, ckpt.data_ptr(), lam.data_ptr(),
                                     gk.data_ptr(), work.data_ptr(), 2, None) == N.ADV_ERR_INVALID_ARG
