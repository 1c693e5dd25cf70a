"""The oracle's discrete adjoints against central finite differences (CPU, FP64).

The adjoint of a step must be the exact transpose of that step, so directional derivatives of
J = 1/2 |u(T) - target|^2 from the adjoint must agree with central differences of J to the
truncation error of the differences (J is smooth in k and u0)."""
import numpy as np
import pytest


def _heatk_case(seed=0, shape=(11, 9, 8), zero_boundary=True):
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    k = np.exp(0.5 * rng.standard_normal(n))
    u0 = rng.random(n)
    if zero_boundary:
        u0.reshape(shape[::-1])[[0, -1], :, :] = 0
    target = rng.random(n)
    h = 1.0 / (max(shape) - 1)
    c = (0.1 / k.max(),) * 3  # dt/h^2 with dt k_max / h^2 = 0.1
    return shape, zero_boundary, c, k, u0, target


@pytest.mark.parametrize("zero_boundary", [True, False])
def test_heatk_adjoint_matches_central_differences(oracle, zero_boundary):
    shape, zb, c, k, u0, target = _heatk_case(1, zero_boundary=zero_boundary)
    steps = 7
    J, gk, gu = oracle.heatk_loss_and_gradient(shape, zb, c, k, u0, target, steps)
    rng = np.random.default_rng(2)
    for _ in range(4):
        dk = rng.standard_normal(k.size)
        du = rng.standard_normal(u0.size)
        eps = 1e-6
        Jp, _, _ = oracle.heatk_loss_and_gradient(shape, zb, c, k + eps * dk, u0 + eps * du, target, steps)
        Jm, _, _ = oracle.heatk_loss_and_gradient(shape, zb, c, k - eps * dk, u0 - eps * du, target, steps)
        fd = (Jp - Jm) / (2 * eps)
        ad = float(np.dot(gk, dk) + np.dot(gu, du))
        assert abs(fd - ad) <= 1e-7 * max(1.0, abs(ad)), (fd, ad)


def test_heatk_step_is_linear_in_u_and_adjoint_is_its_transpose(oracle):
    shape, zb, c, k, _, _ = _heatk_case(3, shape=(6, 5, 7))
    n = k.size
    rng = np.random.default_rng(4)
    u = rng.random(n)
    lam = rng.random(n)
    # <lam, A u> == <A^T lam, u> for the (linear in u) step map
    Au = oracle.heatk_step(shape, zb, c, k, u)
    g = np.zeros(n)
    ATl = oracle.heatk_adjoint(shape, zb, c, k, u, lam, g)
    assert np.dot(lam, Au) == pytest.approx(np.dot(ATl, u), rel=1e-13)


def _burgers_case(n, weno, seed=0):
    from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig
    cfg = BurgersConfig.periodic(n, weno=weno, lf="local")
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) * cfg.dx
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    u0 = (0.5 + 0.3 * np.sin(np.pi * X + 0.3) * np.cos(np.pi * Y) + 0.2 * np.sin(np.pi * Z + 1.0)
          + 0.01 * rng.standard_normal(X.shape))
    u0 = np.ascontiguousarray(u0.transpose(2, 1, 0)).ravel()  # x fastest
    target = u0 + 0.05 * rng.standard_normal(u0.size)
    dt = 0.3 * cfg.dx / np.abs(u0).max()
    return cfg, u0, target, dt


@pytest.mark.parametrize("weno", ["z", "js"])
def test_burgers_adjoint_matches_central_differences(oracle, weno):
    """WENO5-JS is smooth; WENO5-Z has kinks where |beta_0 - beta_2| changes sign, which a finite
    step may cross, so the differences are taken over a small scan of steps and the best one
    must agree (at the smallest steps the kinks are no longer crossed)."""
    cfg, u0, target, dt = _burgers_case(12, weno)
    steps = 4
    J, g = oracle.burgers_loss_and_gradient(cfg, u0, target, dt, steps)
    rng = np.random.default_rng(7)
    for _ in range(3):
        d = rng.standard_normal(u0.size)
        ad = float(np.dot(g, d))
        errs = []
        for eps in (1e-6, 1e-7, 3e-8):
            Jp, _ = oracle.burgers_loss_and_gradient(cfg, u0 + eps * d, target, dt, steps)
            Jm, _ = oracle.burgers_loss_and_gradient(cfg, u0 - eps * d, target, dt, steps)
            errs.append(abs((Jp - Jm) / (2 * eps) - ad))
        assert min(errs) <= 2e-6 * max(1.0, abs(ad)), (errs, ad)
