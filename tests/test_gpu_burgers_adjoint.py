"""Discrete adjoint of the periodic local-LF WENO5 / WENO5-Z SSP-RK3 Burgers step on the GPU.

The kernel (a fused gather over x/y faces in shared memory and z faces in register windows) is
checked against the oracle's independent scatter-form adjoint on the same stage inputs, the
checkpointed backward run against the oracle's gradient from stored states for several checkpoint
intervals, the FP64 gradient against central differences of the FP64 forward run (with a small
scan of steps: WENO5-Z has kinks where |beta_0 - beta_2| changes sign), and the FP32 gradient
against the FP64 one."""
import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig, burgers_adjoint_step, burgers_run_fixed

pytestmark = pytest.mark.gpu


def _state(cfg, seed):
    lib = N.load()
    u = np.empty(cfg.numel)
    N.check(lib.adv_ic_burgers_fourier(cfg.nx, cfg.ny, cfg.nz, 2.0, seed, 16, 0.1,
                                       u.ctypes.data_as(N.C.POINTER(N.C.c_double))), "ic")
    return u


def _cfg(shape, weno, dtype=np.float64):
    nx, ny, nz = shape
    c = BurgersConfig(nx, ny, nz, 2.0 / nx, 2.0 / ny, 2.0 / nz, N.ADV_WENO5_Z if weno == "z" else N.ADV_WENO5_JS,
                      N.ADV_LF_LOCAL, N.ADV_BC_PERIODIC, N.ADV_DIV_FAST)
    return c


def _t(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("shape", [(40, 36, 28), (32, 16, 12), (37, 23, 19)])
@pytest.mark.parametrize("weno", ["z", "js"])
def test_adjoint_step_matches_oracle(cuda, native, oracle, weno, shape):
    import torch
    cfg = _cfg(shape, weno)
    u0 = _state(cfg, 3)
    dt = 0.3 * cfg.dx / np.abs(u0).max()
    states, u1_end = oracle.burgers_forward_states(cfg, u0, dt, 1)
    un, u1, u2 = states[0]
    lam = np.random.default_rng(1).standard_normal(u0.size)
    want = oracle.burgers_step_adjoint(cfg, un, u1, u2, dt, lam)
    for dtype, tol in ((np.float64, 1e-12), (np.float32, 5e-5)):
        d = [_t(a.astype(dtype), cuda) for a in (un, u1, u2, lam)]
        burgers_adjoint_step(cfg, d[0], d[1], d[2], dt, d[3])
        torch.cuda.synchronize()
        got = d[3].double().cpu().numpy()
        assert _rel(got, want) < tol, (dtype, _rel(got, want))


@pytest.mark.parametrize("interval", [1, 3, 7, 10, None])
@pytest.mark.parametrize("weno", ["z", "js"])
def test_checkpointed_gradient_matches_oracle(cuda, native, oracle, weno, interval):
    """interval None: the wrapper's choice (here the whole run kept, nothing recomputed)."""
    import torch
    shape = (24, 20, 18)
    cfg = _cfg(shape, weno)
    u0 = _state(cfg, 5)
    target = _state(cfg, 6)
    steps = 7
    dt = 0.3 * cfg.dx / np.abs(u0).max()
    J, g = oracle.burgers_loss_and_gradient(cfg, u0, target, dt, steps)
    uu = _t(u0, cuda).requires_grad_(True)
    uT = burgers_run_fixed(cfg, uu, dt, steps, interval)
    loss = 0.5 * ((uT - _t(target, cuda)) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    assert abs(loss.item() - J) <= 1e-12 * J
    assert _rel(uu.grad.cpu().numpy(), g) < 1e-11


@pytest.mark.parametrize("steps,interval", [(10, 4), (12, 4), (7, 7), (5, 9), (9, 1), (1, 3)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_backward_with_and_without_the_kept_interval(cuda, native, dtype, steps, interval):
    """adv_burgers_forward leaves its last interval's stage inputs in work; the backward run that
    takes them (ADV_BURGERS_LAST_INTERVAL_IN_WORK) and the one that recomputes them (flags 0) give
    the same bits, for last intervals of every length, and the forward's result is the plain
    run's (no checkpoints)."""
    import torch
    shape = (24, 20, 18)
    cfg = _cfg(shape, "z")
    u0 = _state(cfg, 5).astype(dtype)
    target = _state(cfg, 6).astype(dtype)
    dt = 0.3 * cfg.dx / np.abs(u0).max()
    code = N.ADV_F32 if dtype == np.float32 else N.ADV_F64
    d = cfg.desc(code)
    cb, wb = N.C.c_size_t(0), N.C.c_size_t(0)
    assert native.adv_burgers_checkpoint_bytes(N.C.byref(d), steps, interval, N.C.byref(cb), N.C.byref(wb)) == N.ADV_OK
    plain = _t(u0, cuda)
    w2 = torch.empty(2 * plain.numel() + 256, dtype=plain.dtype, device=cuda)
    assert native.adv_burgers_forward(N.C.byref(d), plain.data_ptr(), dt, steps, interval, None, w2.data_ptr(),
                                      None) == N.ADV_OK
    res = []
    for flags in (N.ADV_BURGERS_LAST_INTERVAL_IN_WORK, 0):
        u = _t(u0, cuda)
        ckpt = torch.empty(cb.value, dtype=torch.uint8, device=cuda)
        work = torch.empty(wb.value, dtype=torch.uint8, device=cuda)
        assert native.adv_burgers_forward(N.C.byref(d), u.data_ptr(), dt, steps, interval, ckpt.data_ptr(),
                                          work.data_ptr(), None) == N.ADV_OK
        assert torch.equal(u, plain)
        lam = u - _t(target, cuda)
        assert native.adv_burgers_backward(N.C.byref(d), dt, steps, interval, ckpt.data_ptr(), lam.data_ptr(),
                                           work.data_ptr(), flags, None) == N.ADV_OK
        torch.cuda.synchronize()
        res.append(lam.cpu().numpy())
    assert np.array_equal(res[0], res[1])
    assert native.adv_burgers_backward(N.C.byref(d), dt, steps, interval, ckpt.data_ptr(), lam.data_ptr(),
                                       work.data_ptr(), 2, None) == N.ADV_ERR_INVALID_ARG


@pytest.mark.parametrize("weno", ["z", "js"])
def test_gradient_matches_central_differences_fp64(cuda, native, weno):
    import torch
    shape = (32, 32, 32)
    cfg = _cfg(shape, weno)
    u0 = _t(_state(cfg, 7), cuda)
    target = _t(_state(cfg, 8), cuda)
    steps = 12
    dt = 0.3 * cfg.dx / u0.abs().max().item()

    def J(u):
        with torch.no_grad():
            return 0.5 * float(((burgers_run_fixed(cfg, u, dt, steps) - target) ** 2).sum())

    uu = u0.clone().requires_grad_(True)
    (0.5 * ((burgers_run_fixed(cfg, uu, dt, steps) - target) ** 2).sum()).backward()
    rng = np.random.default_rng(9)
    for _ in range(4):
        d = _t(rng.standard_normal(u0.numel()), cuda)
        ad = float((uu.grad * d).sum())
        errs = [abs((J(u0 + e * d) - J(u0 - e * d)) / (2 * e) - ad) for e in (1e-7, 1e-8, 1e-9)]
        assert min(errs) <= 1e-5 * abs(ad), (errs, ad)


def test_fp32_gradient_close_to_fp64(cuda, native):
    import torch
    shape = (48, 48, 48)
    cfg = _cfg(shape, "z")
    u0 = _state(cfg, 11)
    target = _state(cfg, 12)
    steps = 20
    dt = 0.3 * cfg.dx / np.abs(u0).max()
    grads = {}
    for dt_ in (torch.float32, torch.float64):
        uu = _t(u0, cuda).to(dt_).requires_grad_(True)
        (0.5 * ((burgers_run_fixed(cfg, uu, dt, steps, 5) - _t(target, cuda).to(dt_)) ** 2).sum()).backward()
        grads[dt_] = uu.grad.double()
    rel = (torch.linalg.vector_norm(grads[torch.float32] - grads[torch.float64])
           / torch.linalg.vector_norm(grads[torch.float64])).item()
    assert rel < 1e-4, rel


def test_adjoint_rejects_other_schemes(cuda, native):
    cfg = BurgersConfig.periodic(16, lf="global")
    d = cfg.desc(N.ADV_F32)
    cb, wb = N.C.c_size_t(0), N.C.c_size_t(0)
    assert native.adv_burgers_checkpoint_bytes(N.C.byref(d), 10, 3, N.C.byref(cb), N.C.byref(wb)) == \
        N.ADV_ERR_UNSUPPORTED
