"""The oracle's restatement of the MATLAB Burgers prototypes (WENO5 / WENO7 residuals and the
LFWENO{5,7}FDM solver loops), pinned against the prototypes themselves: the fixture
tests/golden/matlab_burgers_prototypes.npz holds their outputs, produced by running the
reference's .m files through tests/golden/matlab_subset.py (tests/golden/make_weno_golden.py).
Also: WENO7's order of accuracy, exactness on cubics, and the LSRK(5,4) amplification factor."""
from __future__ import annotations

import ast
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

FIX = Path(__file__).resolve().parent / "golden" / "matlab_burgers_prototypes.npz"


@pytest.fixture(scope="module")
def fx():
    return np.load(FIX)


def _residual_cases():
    z = np.load(FIX)
    out = []
    for k in z.files:
        p = k.split("/")
        if p[0] == "res" and len(p) == 4:
            out.append((p[1], int(p[2][1:]), int(p[3][1:])))
    return out


@pytest.mark.parametrize("name,order,axis", _residual_cases())
def test_residual_equals_matlab_prototype(fx, name, order, axis):
    u = fx[f"res/{name}/u"]
    ref = fx[f"res/{name}/o{order}/a{axis}"]
    got = O.proto_residual(order, axis, u, float(fx["res/h"][axis]), line_max=(u.ndim == 1))
    assert np.array_equal(got, ref)  # same operations in the same order: bit for bit


@pytest.mark.parametrize("order,ndim", [(5, 1), (5, 2), (5, 3), (7, 1), (7, 2), (7, 3)])
def test_solver_loop_equals_matlab_prototype(fx, order, ndim):
    """2D/3D: the drivers' solver loops on small grids; 1D: the whole LFWENO{5,7}FDM1d.m drivers
    (their grid, CFL, tEnd and square-jump initial condition). Bit for bit, same steps and t."""
    k = f"run/o{order}/d{ndim}"
    t_ref, it_ref, cfl, tend, dx = fx[k + "/t_it_cfl_tend_dx"]
    u, t, it = O.proto_run(order, fx[k + "/u0"], [dx] * ndim, float(cfl), float(tend))
    ref = fx[k + "/u"]
    assert it == int(it_ref) and t == t_ref
    assert np.array_equal(u, ref)


def test_fixture_records_the_prototype_calls(fx):
    calls = dict(ast.literal_eval(str(fx["meta/calls"])))  # repr of (name, count) pairs
    assert calls["WENO7resAdv_Z"] > 5 and calls["WENO5resAdv_X"] > 5
    assert "WENO7resAdv_X.m" in str(fx["meta/source_sha256"])


def _cell_average(poly, a, b):
    P = np.polyint(poly)
    return (np.polyval(P, b) - np.polyval(P, a)) / (b - a)


def test_weno7_reproduces_cubics_whatever_the_weights():
    """Each of the four candidates is exact for cubics, so any convex weights give the exact
    face value h(x_{i+1/2}) from the cell averages of h (the finite-difference WENO flux)."""
    rng = np.random.default_rng(7)
    for _ in range(20):
        poly = rng.standard_normal(4)
        dxc = 0.1 + rng.random()
        edges = dxc * (np.arange(8) - 3.5)          # cells i-3..i+3, face i+1/2 at 0.5*dxc
        f = [_cell_average(poly, edges[j], edges[j + 1]) for j in range(7)]
        assert abs(O.weno7_side(f) - np.polyval(poly, edges[4])) <= 1e-12 * (1 + np.max(np.abs(f)))


def test_weno7_linear_weights_are_exact_to_degree_six():
    """Where the smoothness indicators are far below eps (amplitude 1e-10) the weights are the
    linear ones, 1/35, 12/35, 18/35, 4/35, whose combination is the seven-cell reconstruction:
    exact for polynomials of degree 6 (seventh order), not for degree 7. (The weights' distance
    from the linear ones scales with beta/eps ~ amplitude^2: about 1e-10 relative here.)"""
    rng = np.random.default_rng(11)
    amp = 1e-10
    edges = 0.4 * (np.arange(8) - 3.5)
    for degree, exact in ((6, True), (7, False)):
        for _ in range(5):
            poly = amp * rng.standard_normal(degree + 1)
            poly[0] = amp * (1.0 + rng.random())  # leading coefficient well away from 0
            f = [_cell_average(poly, edges[j], edges[j + 1]) for j in range(7)]
            err = abs(O.weno7_side(f) - np.polyval(poly, edges[4]))
            if exact:
                assert err <= 1e-8 * amp
            else:
                assert err >= 1e-3 * amp


def test_weno7_residual_converges_faster_than_weno5():
    """d(u^2/2)/dx of a smooth positive u away from the line ends, per-node split a = |u|."""
    def l1_error(order, n):
        x = np.linspace(-1, 1, n)
        dx = x[1] - x[0]
        u = 1.5 + 0.3 * np.sin(np.pi * x)
        r = O.proto_residual(order, 0, u, dx)
        exact = u * 0.3 * np.pi * np.cos(np.pi * x)
        sl = slice(8, n - 8)
        return np.mean(np.abs(r[sl] - exact[sl]))
    orders = {}
    for order in (5, 7):
        e = [l1_error(order, n) for n in (41, 81, 161)]
        orders[order] = math.log2(e[1] / e[2])
    assert orders[5] > 4.0, orders
    assert orders[7] > 5.8, orders  # 6.2 observed (Jiang-Shu weights lose a little near u' = 0)
    assert l1_error(7, 161) < l1_error(5, 161) / 50


def test_lsrk54_is_fourth_order_in_time():
    """R(z) - sum_{k<=4} z^k/k! = O(z^5): halving z divides the defect by about 32."""
    def defect(z):
        taylor = sum(z ** k / math.factorial(k) for k in range(5))
        return abs(O.lsrk54_gain(z) - taylor)
    for theta in (0.0, 2.0, math.pi):
        z = 0.02 * complex(math.cos(theta), math.sin(theta))
        d1, d2 = defect(z), defect(z / 2)
        assert d1 < 1e-9 and 24 < d1 / d2 < 40
    # stability on the imaginary axis segment the WENO drivers use (CFL 0.4)
    assert abs(O.lsrk54_gain(complex(0.0, 1.0))) <= 1.0
