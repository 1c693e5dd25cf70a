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
        run("c = {1, 2};")  # cell arrays
    with pytest.raises(MatlabError):
        run("a = [1 2]; b = a';")  # transpose
    with pytest.raises(MatlabError):
        run("y = undefined_function(1);")


def test_strings_switch_logic_ranges_and_multiple_outputs():
    e = run("s = 'dont'; switch s\n case 'add'; v = 1;\n case 'dont'; v = 2;\n otherwise\n v = 3;\n end\n"
            "x = -1:0.5:1; k = 0; if (k > 0 && undefined_function(1)) || k == 0, k = 5; end\n"
            "[X, Y] = meshgrid(1:3, 10:10:20); u = zeros(size(X)); u(4) = 7; u(2, 3) = 9;\n"
            "t = sum(x); m = norm([1 -4 2], inf); f = 'L: %1.2e \\n'; fprintf(f, t);")
    assert e["v"] == 2.0 and e["k"] == 5.0 and e["t"] == 0.0 and e["m"] == 4.0
    np.testing.assert_array_equal(e["x"], [[-1.0, -0.5, 0.0, 0.5, 1.0]])
    np.testing.assert_array_equal(e["X"], [[1, 2, 3], [1, 2, 3]])
    np.testing.assert_array_equal(e["Y"], [[10, 10, 10], [20, 20, 20]])
    np.testing.assert_array_equal(e["u"], [[0, 0, 0], [0, 7, 9]])  # linear index 4 = (2, 2), column-major


def test_function_files_with_several_outputs(tmp_path):
    (tmp_path / "twoout.m").write_text("function [s, p] = twoout(a, b)\n% sum and product\ns = a + b;\np = a * b;\n")
    it = Interpreter(tmp_path)
    env = it.run("[a, b] = twoout(3, 4); c = twoout(1, 2);", {})
    assert (env["a"], env["b"], env["c"]) == (7.0, 12.0, 3.0)
    assert it.call_file("twoout", [2.0, 5.0], nargout=2) == [7.0, 10.0]


def test_if_elseif_else():
    e = run("for k = 1:3\n if k == 1, a = 1; elseif k == 2\n b = 2; else\n c = 3; end\n end")
    assert (e["a"], e["b"], e["c"]) == (1.0, 2.0, 3.0)


def test_end_in_indices_command_syntax_and_pulses():
    e = run("clear; close all; clc;\nx = [3 5 7 9]; a = x(end); b = x(end-1); m = min(x);\n"
            "p = rectangularPulse(4, 8, [3 4 5 8 9]);")
    assert (e["a"], e["b"], e["m"]) == (9.0, 7.0, 3.0)
    np.testing.assert_array_equal(e["p"], [[0.0, 0.5, 1.0, 0.5, 0.0]])
