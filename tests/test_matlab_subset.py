"""The MATLAB-subset interpreter that produces the prototype fixtures (tests/golden/
matlab_subset.py): MATLAB's semantics for the constructs the prototypes use, checked on
snippets with known answers, and a refusal for anything outside the subset."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from matlab_subset import Interpreter, MatlabError  # noqa: E402


def run(src, **env):
    return Interpreter().run(src, dict(env))


def test_precedence_and_ranges():
    e = run("a = -2.^2; b = 2*3+4/2; c = 4:(2+3); d = (1+2)*3; f = 12/35;")
    assert e["a"] == -4.0 and e["b"] == 8.0 and e["d"] == 9.0 and e["f"] == 12 / 35
    np.testing.assert_array_equal(e["c"], [[4.0, 5.0]])


def test_row_literals_split_on_signs_like_matlab():
    e = run("r = [ 1.0 ...\n -2.0/4.0 ...\n 3 - 1 4-1, 5];")
    np.testing.assert_array_equal(e["r"], [[1.0, -0.5, 2.0, 3.0, 5.0]])


def test_one_based_indexing_colon_and_linear_order():
    a = np.arange(24, dtype=float).reshape(2, 3, 4)
    e = run("b = a(:, 2, :); c = a(2, [1 3], 4); d = a(:); s = size(a);", a=a)
    np.testing.assert_array_equal(e["b"], a[:, 1:2, :])
    np.testing.assert_array_equal(e["c"], [[a[1, 0, 3], a[1, 2, 3]]])
    np.testing.assert_array_equal(e["d"].ravel(), a.ravel(order="F"))  # column-major
    np.testing.assert_array_equal(e["s"], [[2, 3, 4]])


def test_cat_and_indexed_assignment():
    w = np.arange(6, dtype=float).reshape(2, 3)
    e = run("W = cat(2, w(:,1,:), w(:,1,:), w, w(:,3,:)); h = zeros(size(W)); I = 2:3; h(:,I,:) = W(:,I,:) * 2;",
            w=w)
    np.testing.assert_array_equal(e["W"], np.hstack([w[:, :1], w[:, :1], w, w[:, 2:]]))
    expect = np.zeros((2, 6))
    expect[:, 1:3] = 2 * e["W"][:, 1:3]
    np.testing.assert_array_equal(e["h"], expect)


def test_control_flow_handles_and_builtins():
    e = run("f = @(w) w.^2/2; t = 0; it = 0; while t < 1, t = t + 0.3; it = it + 1; end\n"
            "s = 0; for k = 1:4\n s = s + k; if rem(k,2)==0, s = s + 10; end\n end\n"
            "m = max(abs([-3 2])); g = f(3); surf(x, y, u); drawnow;")
    assert e["it"] == 4 and e["s"] == 30.0 and e["m"] == 3.0 and e["g"] == 4.5


def test_outside_the_subset_is_refused():
    with pytest.raises(MatlabError):
        run("a = [1 2; 3 4] * [1 2; 3 4];")
    with pytest.raises(MatlabError):
        run("x = 0:0.5:2;")
    with pytest.raises(MatlabError):
        run("s = 'text';")
    with pytest.raises(MatlabError):
        run("y = undefined_function(1);")
