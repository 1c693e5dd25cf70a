"""Batched ensembles (adv_ensemble_*) against per-member runs of the single-problem entry points.

Every member of an ensemble must end bit for bit where adv_heat_run / adv_burgers_run would take
it on its own (same stage kernels' arithmetic, same per-member dt and Lax-Friedrichs constants,
same stop test), whether the run goes through the ensemble's CUDA graph or through direct
launches, with uneven member sizes, with FP32 heat members in tiles of two widths in one launch,
with members whose rows TMA cannot describe (the whole batch then takes the cp.async path), and
with heat and Burgers members running concurrently.
"""
import ctypes as C

import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import (BurgersConfig, Ensemble, HeatConfig, burgers_run,
                                                       heat_run)

pytestmark = pytest.mark.gpu


def _heat_cfg(nx, ny, nz, k, scheme, order=2):
    """O2 Dirichlet heat with r = k dt / h^2 = 1/8 on h = 1/(max n - 1); O4 with r = 1/16."""
    h = 1.0 / (max(nx, ny, nz) - 1)
    if order == 2:
        c = k / (h * h)
        return HeatConfig(3, nx, ny, nz, 2, 1, True, c, c, c, 0.125 * h * h / k, scheme)
    c = k / (12 * h * h)
    return HeatConfig(3, nx, ny, nz, 4, 2, False, c, c, c, 0.0625 * h * h / k, scheme)


def _heat_state(cfg, dtype, seed, cuda):
    import torch
    rng = np.random.default_rng(seed)
    return torch.from_numpy(rng.random(cfg.numel).astype(dtype)).to(cuda)


def _burgers_state(cfg, dtype, seed, cuda):
    import torch
    lib = N.load()
    u = np.empty(cfg.numel)
    N.check(lib.adv_ic_burgers_fourier(cfg.nx, cfg.ny, cfg.nz, cfg.dx * cfg.nx, seed, 8, 0.1,
                                       u.ctypes.data_as(C.POINTER(C.c_double))), "ic")
    return torch.from_numpy(u.astype(dtype)).to(cuda)


HEAT_SETS = {
    "aligned": [(64, 48, 40), (96, 96, 96), (36, 20, 70), (128, 64, 33), (8, 8, 9)],
    "unaligned": [(64, 48, 40), (37, 29, 31), (96, 40, 17)],  # nx = 37: 148-byte rows
    # FP32 members in 128-wide tiles (nx 128, 96) and 64-wide tiles (nx 160, 64, 192, 40): one
    # launch runs both widths (heat_batch_mixed_kernel), the table reordered by width
    "widths": [(160, 24, 20), (64, 40, 17), (128, 33, 12), (192, 20, 9), (40, 16, 30), (96, 20, 11)],
    "narrow": [(64, 40, 17), (40, 16, 30), (192, 20, 9)],  # 64-wide tiles only
}


@pytest.mark.parametrize("direct", [False, True], ids=["graph", "direct"])
@pytest.mark.parametrize("scheme,steps", [(N.ADV_EULER, 7), (N.ADV_EULER, 6), (N.ADV_SSPRK3, 4)],
                         ids=["euler-odd", "euler-even", "rk3"])
@pytest.mark.parametrize("sizes", ["aligned", "unaligned", "widths", "narrow"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_heat_ensemble_matches_per_member_runs(cuda, native, dtype, sizes, scheme, steps, direct):
    rng = np.random.default_rng(5)
    cfgs = [_heat_cfg(*s, k=float(10 ** rng.uniform(-1, 1)), scheme=scheme) for s in HEAT_SETS[sizes]]
    us = [_heat_state(c, dtype, 100 + i, cuda) for i, c in enumerate(cfgs)]
    refs = [u.clone() for u in us]
    ens = Ensemble(heat=list(zip(cfgs, us)), heat_time=scheme)
    ens.run(steps, direct=direct)
    for c, r in zip(cfgs, refs):
        heat_run(c, r, steps)
    import torch
    torch.cuda.synchronize()
    for i, (u, r) in enumerate(zip(us, refs)):
        assert torch.equal(u, r), f"member {i} {HEAT_SETS[sizes][i]}"
    sh = ens.shape()
    assert sh["heat_units"] > 0 and sh["heat_ctas"] >= 1
    ens.close()


def test_heat_ensemble_order4_and_repeated_runs(cuda, native):
    import torch
    cfgs = [_heat_cfg(40, 36, 33, 1.0, N.ADV_SSPRK3, order=4), _heat_cfg(64, 64, 48, 3.0, N.ADV_SSPRK3, order=4)]
    us = [_heat_state(c, np.float64, 7 + i, cuda) for i, c in enumerate(cfgs)]
    refs = [u.clone() for u in us]
    ens = Ensemble(heat=list(zip(cfgs, us)), heat_time=N.ADV_SSPRK3)
    ens.run(3)
    ens.run(2)  # continues from the state the first run left
    for c, r in zip(cfgs, refs):
        heat_run(c, r, 5)
    torch.cuda.synchronize()
    for u, r in zip(us, refs):
        assert torch.equal(u, r)
    ens.close()


def _burgers_members(dtype, div, cuda):
    cfgs = [BurgersConfig.periodic(32, div=div), BurgersConfig.periodic(48, div=div),
            BurgersConfig(40, 36, 28, 2 / 40, 2 / 36, 2 / 28, N.ADV_WENO5_Z, N.ADV_LF_GLOBAL, N.ADV_BC_PERIODIC, div),
            BurgersConfig(37, 33, 30, 0.05, 0.05, 0.05, N.ADV_WENO5_Z, N.ADV_LF_LOCAL, N.ADV_BC_FROZEN, div),
            BurgersConfig(72, 40, 1, 2 / 72, 2 / 40, 2 / 72, N.ADV_WENO5_Z, N.ADV_LF_GLOBAL, N.ADV_BC_PERIODIC, div)]
    ends = [0.05, 0.12, 0.08, 0.1, 0.15]
    us = [_burgers_state(c, dtype, 11 + i, cuda) for i, c in enumerate(cfgs)]
    return cfgs, ends, us


@pytest.mark.parametrize("direct", [False, True], ids=["graph", "direct"])
@pytest.mark.parametrize("dtype,div", [(np.float32, N.ADV_DIV_FAST), (np.float32, N.ADV_DIV_F64),
                                       (np.float64, N.ADV_DIV_F32), (np.float64, N.ADV_DIV_FAST)],
                         ids=["f32-fast", "f32-div64", "f64", "f64-fast"])
def test_burgers_ensemble_matches_per_member_runs(cuda, native, dtype, div, direct):
    import torch
    cfgs, ends, us = _burgers_members(dtype, div, cuda)
    refs = [u.clone() for u in us]
    ens = Ensemble(burgers=[(c, u, te, 0.4) for c, u, te in zip(cfgs, us, ends)])
    ens.run(0, direct=direct)
    for i, (c, r, te) in enumerate(zip(cfgs, refs, ends)):
        t, steps = burgers_run(c, r, te, 0.4)
        te_, steps_ = ens.burgers_result(i)
        assert steps_ == steps and te_ == t, (i, steps_, steps, te_, t)
    torch.cuda.synchronize()
    for i, (u, r) in enumerate(zip(us, refs)):
        assert torch.equal(u, r), f"member {i}"
    ens.close()


def test_burgers_ensemble_viscous_fixed_dt_and_step_limits(cuda, native):
    """The reference scheme (frozen layers, local LF, viscous term, fixed dt) with per-member
    step limits: members stop at their own max_steps while the others go on."""
    import torch
    cfgs = [BurgersConfig.reference(2, 2, 2, 40, 36, 33), BurgersConfig.reference(2, 2, 2, 33, 40, 36)]
    us = [_burgers_state(c, np.float64, 3 + i, cuda) for i, c in enumerate(cfgs)]
    refs = [u.clone() for u in us]
    limits = [3, 1 << 40]
    ens = Ensemble(burgers=[(c, u, 0.06, 0.3, N.ADV_DT_FIXED, m) for c, u, m in zip(cfgs, us, limits)])
    ens.run(0)
    for i, (c, r) in enumerate(zip(cfgs, refs)):
        t, steps = burgers_run(c, r, 0.06, 0.3, dt_rule=N.ADV_DT_FIXED, max_steps=limits[i])
        assert ens.burgers_result(i) == (t, steps)
    assert ens.burgers_result(0)[1] == 3
    torch.cuda.synchronize()
    for u, r in zip(us, refs):
        assert torch.equal(u, r)
    ens.close()


def test_mixed_ensemble_runs_both_loops(cuda, native):
    import torch
    hcfgs = [_heat_cfg(64, 64, 64, 0.3, N.ADV_EULER), _heat_cfg(96, 80, 72, 5.0, N.ADV_EULER),
             _heat_cfg(32, 40, 48, 1.0, N.ADV_EULER)]
    hus = [_heat_state(c, np.float32, 20 + i, cuda) for i, c in enumerate(hcfgs)]
    bcfgs = [BurgersConfig.periodic(32, div="fast"), BurgersConfig.periodic(64, div="fast")]
    bus = [_burgers_state(c, np.float32, 30 + i, cuda) for i, c in enumerate(bcfgs)]
    hrefs = [u.clone() for u in hus]
    brefs = [u.clone() for u in bus]
    ens = Ensemble(heat=list(zip(hcfgs, hus)), burgers=[(c, u, 0.1, 0.4) for c, u in zip(bcfgs, bus)])
    before = N.load().adv_kernel_launch_count()
    ens.run(25)
    launched = N.load().adv_kernel_launch_count() - before
    for c, r in zip(hcfgs, hrefs):
        heat_run(c, r, 25)
    steps = []
    for i, (c, r) in enumerate(zip(bcfgs, brefs)):
        t, s = burgers_run(c, r, 0.1, 0.4)
        assert ens.burgers_result(i) == (t, s)
        steps.append(s)
    torch.cuda.synchronize()
    for u, r in zip(hus + bus, hrefs + brefs):
        assert torch.equal(u, r)
    # 12 heat iterations of tick + 2 stages, one odd step, 2 max|u| launches, Burgers steps x 4
    assert launched == 12 * 3 + 1 + 2 + 4 * max(steps)
    ens.close()


def test_ensemble_rejects_mixed_members(cuda, native):
    import torch
    a = _heat_cfg(16, 16, 16, 1.0, N.ADV_EULER)
    u32 = torch.zeros(a.numel, device=cuda)
    u64 = torch.zeros(a.numel, device=cuda, dtype=torch.float64)
    with pytest.raises(N.AdvError) as ei:
        Ensemble(heat=[(a, u32), (a, u64)])
    assert ei.value.status == N.ADV_ERR_INVALID_ARG
    assert b"share dtype" in N.load().adv_last_error_string()
    flat = HeatConfig.dirichlet_o2(2, 16)
    with pytest.raises(N.AdvError):
        Ensemble(heat=[(flat, torch.zeros(flat.numel, device=cuda))])
    b1, b2 = BurgersConfig.periodic(16, weno="z"), BurgersConfig.periodic(16, weno="js")
    with pytest.raises(N.AdvError):
        Ensemble(burgers=[(b1, torch.zeros(b1.numel, device=cuda), 0.1, 0.4),
                          (b2, torch.zeros(b2.numel, device=cuda), 0.1, 0.4)])
