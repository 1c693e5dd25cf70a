"""Fused Burgers WENO stage and the graph-resident time loop on the GPU against the oracle.
FP64 state (reference operand order) is bit-exact; FP32 state (one division per WENO side) is
held to a stated tolerance against the FP32 and FP64 oracles."""
import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig, burgers_run, burgers_stage

pytestmark = pytest.mark.gpu


def _t(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def _cases():
    out = []
    for size in [(32, 32, 24), (37, 35, 23), (64, 16, 40)]:
        for weno in (N.ADV_WENO5_Z, N.ADV_WENO5_JS):
            out.append(("periodic-global", size, weno))
            out.append(("periodic-local", size, weno))
            out.append(("frozen-visc", size, weno))
    out.append(("frozen-visc-b2", (24, 22, 40), N.ADV_WENO5_Z))
    out.append(("frozen-local", (40, 20, 12), N.ADV_WENO5_Z))
    return out


def _cfg(kind, size, weno):
    nx, ny, nz = size
    if kind.startswith("periodic"):
        c = BurgersConfig(nx, ny, nz, 2.0 / nx, 2.0 / ny, 2.0 / nz, weno,
                          N.ADV_LF_GLOBAL if kind.endswith("global") else N.ADV_LF_LOCAL, N.ADV_BC_PERIODIC)
    else:
        c = BurgersConfig.reference(2.0, 2.0, 2.0, nx, ny, nz, C=1e-2 if "visc" in kind else 0.0,
                                    bug_b2="b2" in kind)
        c.weno = weno
    return c


def _field(cfg, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 2, cfg.nx, endpoint=False)[None, None, :]
    y = np.linspace(0, 2, cfg.ny, endpoint=False)[None, :, None]
    z = np.linspace(0, 2, cfg.nz, endpoint=False)[:, None, None]
    u = 0.5 + 0.4 * np.sin(np.pi * x + 1) * np.cos(np.pi * y) + 0.3 * np.sin(np.pi * z + 0.5)
    return (u + 0.05 * rng.standard_normal(u.shape)).ravel()


@pytest.mark.parametrize("kind,size,weno", _cases())
@pytest.mark.parametrize("stage", [1, 2, 3])
def test_burgers_stage_fp64_bitwise(cuda, oracle, kind, size, weno, stage):
    cfg = _cfg(kind, size, weno)
    uin = _field(cfg, stage)
    un = uin if stage == 1 else _field(cfg, 100 + stage)
    dt = 1e-3
    want = oracle.burgers_stage(cfg, stage, uin, un, dt)
    a = _t(uin, cuda)
    b = a if stage == 1 else _t(un, cuda)
    out = a.new_full(a.shape, np.nan)
    alpha = float(np.abs(uin).max())
    burgers_stage(cfg, stage, a, b, out, dt, alpha)
    np.testing.assert_array_equal(out.cpu().numpy(), want)


@pytest.mark.parametrize("kind,size,weno", _cases()[:6])
@pytest.mark.parametrize("div", [N.ADV_DIV_F32, N.ADV_DIV_F64, N.ADV_DIV_FAST])
def test_burgers_stage_fp32(cuda, oracle, kind, size, weno, div):
    """FP32 stage vs the FP32 oracle: max |diff| <= 4e-7 * max|u| (a few ulps of the state)."""
    cfg = _cfg(kind, size, weno)
    cfg.div = div
    uin = _field(cfg, 7).astype(np.float32)
    un = _field(cfg, 8).astype(np.float32)
    want = oracle.burgers_stage(cfg, 2, uin, un, 2e-3)
    a, b = _t(uin, cuda), _t(un, cuda)
    out = a.new_full(a.shape, np.nan)
    burgers_stage(cfg, 2, a, b, out, 2e-3, float(np.abs(uin).max()))
    got = out.cpu().numpy()
    assert np.isfinite(got).all()
    assert np.abs(got - want).max() <= 4e-7 * np.abs(want).max()


@pytest.mark.parametrize("kind,size,weno", _cases()[:6] + _cases()[-2:])
def test_burgers_stage_fp64_fast(cuda, oracle, kind, size, weno):
    """FP64 state with ADV_DIV_FAST (common-denominator WENO weights, one division per side, FMAs)
    vs the FP64 oracle's reference operand order: max |diff| <= 1e-14 * max|u|."""
    cfg = _cfg(kind, size, weno)
    cfg.div = N.ADV_DIV_FAST
    uin, un = _field(cfg, 17), _field(cfg, 18)
    want = oracle.burgers_stage(cfg, 2, uin, un, 2e-3)
    a, b = _t(uin, cuda), _t(un, cuda)
    out = a.new_full(a.shape, np.nan)
    burgers_stage(cfg, 2, a, b, out, 2e-3, float(np.abs(uin).max()))
    got = out.cpu().numpy()
    assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max()
    assert not np.array_equal(got, want)  # really the other form


@pytest.mark.parametrize("t_end,tol", [(0.3, 1e-12), (0.6, 1e-10)], ids=["smooth", "shocks"])
def test_burgers_run_fp64_fast_vs_oracle(cuda, oracle, t_end, tol):
    """FP64 fast form over a whole run: same step count; rel-L2 vs the FP64 oracle within tol
    (the shocks of t = 0.6 amplify rounding differences through the nonlinear weights)."""
    cfg = BurgersConfig.periodic(32, weno="z", div="fast")
    u0 = oracle.ic_burgers_fourier(32, 32, 32, 2.0, 3)
    want, t_w, it_w = oracle.burgers_run(cfg, u0, t_end, 0.4, 1)
    u = _t(u0, cuda)
    t, it = burgers_run(cfg, u, t_end, 0.4, N.ADV_DT_MAXU)
    assert it == it_w and t == pytest.approx(t_w, abs=1e-14)
    got = u.cpu().numpy()
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= tol


def test_burgers_stage_reports_max_abs(cuda, oracle):
    import torch
    cfg = _cfg("periodic-global", (32, 32, 24), N.ADV_WENO5_Z)
    u = _field(cfg, 3)
    a = _t(u, cuda)
    out = torch.empty_like(a)
    key = torch.zeros(1, dtype=torch.int64, device=cuda)
    burgers_stage(cfg, 1, a, a, out, 1e-3, float(np.abs(u).max()), maxabs_key=key)
    assert key.view(torch.float64).item() == out.abs().max().item()


@pytest.mark.parametrize("weno", [N.ADV_WENO5_Z, N.ADV_WENO5_JS])
def test_burgers_run_periodic_fp64_bitwise(cuda, oracle, weno):
    """Device-driven loop (dt = CFL dx / max|u^n|, global LF from the fused max|u| reduction, t in
    FP64, while-conditional CUDA graph) reproduces the oracle's loop exactly."""
    cfg = BurgersConfig.periodic(24, weno="z" if weno == N.ADV_WENO5_Z else "js")
    u0 = oracle.ic_burgers_fourier(24, 24, 24, 2.0, 3)
    want, t_w, it_w = oracle.burgers_run(cfg, u0, 0.3, 0.4, 1)
    u = _t(u0, cuda)
    t, it = burgers_run(cfg, u, 0.3, 0.4, N.ADV_DT_MAXU)
    assert it == it_w and t == t_w
    np.testing.assert_array_equal(u.cpu().numpy(), want)


def test_burgers_run_reference_scheme_fp64_bitwise(cuda, oracle):
    """Reference scheme (node grid, local LF, WENO5-Z, C = 1e-5 viscosity with the doubled slabs,
    fixed dt = CFL dx) at 40^3 to t = 0.02."""
    cfg = BurgersConfig.reference(2.0, 2.0, 2.0, 40, 40, 40, C=1e-5, bug_b2=True)
    u0 = oracle.ic_burgers_ref(40, 40, 40, cfg.dx, cfg.dy, cfg.dz)
    want, t_w, it_w = oracle.burgers_run(cfg, u0, 0.02, 0.3, 0, C_visc=1e-5)
    u = _t(u0, cuda)
    t, it = burgers_run(cfg, u, 0.02, 0.3, N.ADV_DT_FIXED)
    assert it == it_w and t == t_w
    np.testing.assert_array_equal(u.cpu().numpy(), want)


@pytest.mark.parametrize("div", [N.ADV_DIV_F32, N.ADV_DIV_F64, N.ADV_DIV_FAST])
def test_burgers_run_fp32_vs_fp64_oracle(cuda, oracle, div):
    """FP32 state to t = 0.5 (past shock formation) within 1e-5 relative L2 of the FP64 oracle."""
    cfg = BurgersConfig.periodic(48, weno="z")
    cfg.div = div
    u0 = oracle.ic_burgers_fourier(48, 48, 48, 2.0, 3)
    want, _, it_w = oracle.burgers_run(cfg, u0, 0.5, 0.4, 1)
    u = _t(u0.astype(np.float32), cuda)
    _, it = burgers_run(cfg, u, 0.5, 0.4, N.ADV_DT_MAXU)
    assert abs(it - it_w) <= 1
    got = u.cpu().numpy().astype(np.float64)
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert rel <= 1e-5, rel


def test_burgers_config_c3_full_size_invariants(cuda, oracle):
    """256^3 periodic WENO5-Z, global LF, CFL 0.4, t = 0.5 in FP32: conserves sum(u) to 1e-6 relative,
    stays finite and bounded by the initial extremes (1e-3 slack for WENO overshoot), and its first
    stage is within 1e-6 of the oracle."""
    import torch
    n = 256
    cfg = BurgersConfig.periodic(n, weno="z")
    u0 = oracle.ic_burgers_fourier(n, n, n, 2.0, 3)
    first = oracle.burgers_stage(cfg, 1, u0.astype(np.float32), u0.astype(np.float32), 1e-3)
    a = _t(u0.astype(np.float32), cuda)
    out = torch.empty_like(a)
    burgers_stage(cfg, 1, a, a, out, 1e-3, float(np.abs(u0.astype(np.float32)).max()))
    assert (out.cpu().numpy() - first).__abs__().max() <= 1e-6 * np.abs(first).max()
    u = _t(u0.astype(np.float32), cuda)
    s0 = u.double().sum().item()
    t, it = burgers_run(cfg, u, 0.5, 0.4, N.ADV_DT_MAXU)
    assert t == pytest.approx(0.5, abs=1e-12) and it > 0
    assert torch.isfinite(u).all().item()
    assert abs(u.double().sum().item() - s0) <= 1e-6 * abs(s0)
    assert u.max().item() <= u0.max() + 1e-3 and u.min().item() >= u0.min() - 1e-3


@pytest.mark.parametrize("weno", ["z", "js"])
def test_fp64_weight_division_equals_ieee_fp32_division(cuda, oracle, weno):
    """With an FP32 state, ADV_DIV_F64 divides each side's two FP32 weight sums in FP64 and rounds the
    quotient to FP32; ADV_DIV_F32 divides them in IEEE FP32. Rounding twice is harmless when the
    wider format carries p >= 2q + 2 bits (53 >= 2*24 + 2; S. Figueroa, "When is double rounding
    innocuous?", 1995), so the two give the same bits: checked on a stage with partial tiles and on
    a run past shock formation."""
    import torch
    cfg32 = BurgersConfig.periodic(48, weno=weno, div="f32")
    cfg64 = BurgersConfig.periodic(48, weno=weno, div="f64")
    u0 = oracle.ic_burgers_fourier(48, 48, 48, 2.0, 3).astype(np.float32)
    a, b = _t(u0, cuda), _t(u0, cuda)
    ta, ia = burgers_run(cfg32, a, 0.5, 0.4, N.ADV_DT_MAXU)
    tb, ib = burgers_run(cfg64, b, 0.5, 0.4, N.ADV_DT_MAXU)
    assert (ta, ia) == (tb, ib) and torch.equal(a, b)
    nx, ny, nz = 37, 35, 23
    for lf in ("global", "local"):
        c32 = BurgersConfig(nx, ny, nz, 2.0 / nx, 2.0 / ny, 2.0 / nz, cfg32.weno,
                            N.ADV_LF_GLOBAL if lf == "global" else N.ADV_LF_LOCAL, N.ADV_BC_PERIODIC, N.ADV_DIV_F32)
        c64 = BurgersConfig(nx, ny, nz, 2.0 / nx, 2.0 / ny, 2.0 / nz, cfg32.weno, c32.lf, N.ADV_BC_PERIODIC,
                            N.ADV_DIV_F64)
        x = _t(np.random.default_rng(5).standard_normal(nx * ny * nz).astype(np.float32), cuda)
        o32, o64 = torch.empty_like(x), torch.empty_like(x)
        burgers_stage(c32, 1, x, x, o32, 1e-3, float(x.abs().max()))
        burgers_stage(c64, 1, x, x, o64, 1e-3, float(x.abs().max()))
        assert torch.equal(o32, o64)


_C3_FP64 = {}


def _c3_fp64(cuda, oracle, weno):
    """The C3 problem (256^3 periodic, global LF, CFL 0.4, max|u| dt, t = 0.5) run with FP64 state
    in the reference's operand order -- the GPU path that equals the FP64 oracle bit for bit
    (test_burgers_run_fp64_bitwise) -- computed once per WENO flavour."""
    if weno not in _C3_FP64:
        n = 256
        cfg = BurgersConfig.periodic(n, weno=weno)
        cfg.div = N.ADV_DIV_F32  # FP64 state: the reference's literal form, bit-exact
        u = _t(oracle.ic_burgers_fourier(n, n, n, 2.0, 3), cuda)
        t, it = burgers_run(cfg, u, 0.5, 0.4, N.ADV_DT_MAXU)
        _C3_FP64[weno] = (u.cpu().numpy(), t, it)
    return _C3_FP64[weno]


# relative L2 bounds of the FP32 state against FP64 at C3's full size. WENO5-Z meets the 1e-5 bar
# with either division (measured 2.5e-6 with the FP64 / IEEE division). WENO5-JS does not, with
# either: its weights d_k / (eps + beta_k)^2 with eps = 1e-6 amplify the FP32 rounding of the
# smoothness indicators where the field is smooth, and the difference grows through the shocks --
# measured 2.7e-4 (FP64 division) and 3.2e-4 (fast division) -- so its bound here is 1e-3
_C3_BOUND = {("z", N.ADV_DIV_F64): 1e-5, ("js", N.ADV_DIV_F64): 1e-3, ("z", N.ADV_DIV_FAST): 1e-5,
             ("js", N.ADV_DIV_FAST): 1e-3}


@pytest.mark.parametrize("weno", ["z", "js"])
@pytest.mark.parametrize("div", [N.ADV_DIV_FAST, N.ADV_DIV_F64])
def test_burgers_config_c3_full_size_fp32_vs_fp64(cuda, oracle, weno, div):
    """C3 at its own size: 256^3 periodic WENO5-Z (and JS), global LF, CFL 0.4, run past shock
    formation to t = 0.5 in FP32 -- with the FP64 weight division (bit-identical to IEEE FP32
    division, test above) and with the reciprocal-based fast division -- against the same run in
    FP64: same step count, relative L2 within the bounds above."""
    n = 256
    want, t_w, it_w = _c3_fp64(cuda, oracle, weno)
    cfg = BurgersConfig.periodic(n, weno=weno)
    cfg.div = div
    u = _t(oracle.ic_burgers_fourier(n, n, n, 2.0, 3).astype(np.float32), cuda)
    t, it = burgers_run(cfg, u, 0.5, 0.4, N.ADV_DT_MAXU)
    assert it == it_w and t == pytest.approx(t_w, abs=1e-12)
    got = u.cpu().numpy().astype(np.float64)
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert rel <= _C3_BOUND[(weno, div)], rel


def test_burgers_run_honours_max_steps(cuda, oracle):
    cfg = BurgersConfig.periodic(16, weno="z")
    u0 = oracle.ic_burgers_fourier(16, 16, 16, 2.0, 3)
    want, t_w, it_w = oracle.burgers_run(cfg, u0, 1.0, 0.4, 1, max_steps=5)
    u = _t(u0, cuda)
    t, it = burgers_run(cfg, u, 1.0, 0.4, N.ADV_DT_MAXU, max_steps=5)
    assert it == 5 == it_w and t == t_w
    np.testing.assert_array_equal(u.cpu().numpy(), want)


def test_burgers_nonfinite_detected(cuda, oracle):
    """A NaN in the state stops the device loop with ADV_ERR_NONFINITE (host-made failure)."""
    cfg = BurgersConfig.periodic(16, weno="z")
    u0 = oracle.ic_burgers_fourier(16, 16, 16, 2.0, 3)
    u0[123] = np.nan
    u = _t(u0, cuda)
    with pytest.raises(N.AdvError) as e:
        burgers_run(cfg, u, 0.1, 0.4, N.ADV_DT_MAXU)
    assert e.value.status == N.ADV_ERR_NONFINITE
