"""The launch-shape autotuner: it picks one of its candidates, never slower than the default it
measured, and a tuned launch gives exactly the results of the default one (the shape only moves
work between CTAs)."""
import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import (BurgersConfig, HeatConfig, HeatKConfig, autotune_burgers,
                                                       autotune_clear, autotune_heat, autotune_heatk, burgers_run,
                                                       heat_run, heatk_run)

pytestmark = pytest.mark.gpu


def _check(r, a_set, b_set):
    assert r["param_a"] in a_set and r["param_b"] in b_set
    assert r["candidates"] == len(a_set) * len(b_set) or r["candidates"] >= len(b_set)
    assert 0 < r["best_us"] <= r["default_us"] * (1 + 1e-9)


def test_heat_tuned_equals_default(cuda, native, oracle):
    import torch
    autotune_clear()
    cfg = HeatConfig.dirichlet_o2(3, 96)
    u0 = torch.from_numpy(oracle.ic_heat3d_blobs(96, 96, 96, 2).astype(np.float32)).to(cuda)
    a = u0.clone()
    heat_run(cfg, a, 11)
    r = autotune_heat(cfg, u0)
    _check(r, set(range(1, 9)), {4, 8, 16, 32})
    b = u0.clone()
    heat_run(cfg, b, 11)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    autotune_clear()


def test_burgers_tuned_equals_default(cuda, native, oracle):
    import torch
    autotune_clear()
    cfg = BurgersConfig.periodic(64, div="fast")
    u0 = torch.from_numpy(oracle.ic_burgers_fourier(64, 64, 64, 2.0, 3).astype(np.float32)).to(cuda)
    a = u0.clone()
    ta = burgers_run(cfg, a, 0.05, 0.4)
    r = autotune_burgers(cfg, u0)
    _check(r, set(range(1, 5)), {4, 8, 16, 32})
    b = u0.clone()
    tb = burgers_run(cfg, b, 0.05, 0.4)
    torch.cuda.synchronize()
    assert ta == tb and torch.equal(a, b)
    autotune_clear()


def test_heatk_tuned_equals_default(cuda, native):
    import torch
    autotune_clear()
    rng = np.random.default_rng(0)
    n = 48
    k = torch.from_numpy(np.exp(0.3 * rng.standard_normal(n ** 3)).astype(np.float32)).to(cuda)
    u0 = torch.from_numpy(rng.random(n ** 3).astype(np.float32)).to(cuda)
    cfg = HeatKConfig.cube(n, 0.12, float(k.max()))

    def grads():
        kk = k.clone().requires_grad_(True)
        uu = u0.clone().requires_grad_(True)
        uT = heatk_run(cfg, kk, uu, 9, 4)
        (0.5 * (uT ** 2).sum()).backward()
        return uT.detach(), kk.grad, uu.grad

    before = grads()
    r1, r2 = autotune_heatk(cfg, k, u0)
    for r in (r1, r2):
        _check(r, {4, 8, 16}, {4, 8, 16, 32})
    after = grads()
    torch.cuda.synchronize()
    for x, y in zip(before, after):
        assert torch.equal(x, y)
    autotune_clear()


def test_autotune_rejects_bad_descriptor(cuda, native):
    r = N.TuneResult()
    bad = N.HeatDesc(4, 8, 8, 8, N.ADV_F32, 2, 1, 1, 1.0, 1.0, 1.0, 0.1)
    assert native.adv_autotune_heat(N.C.byref(bad), None, None, N.C.byref(r)) == N.ADV_ERR_INVALID_ARG
