"""A small interpreter for the subset of MATLAB used by the reference's Burgers prototypes.

Fixture generation only (see make_weno_golden.py and make_heat_golden.py). It runs, on numpy
arrays, the prototype files Matlab_Prototipes/InviscidBurgersNd/WENO{5,7}resAdv_{X,Y,Z,1d}.m,
the solver-loop sections of LFWENO{5,7}FDM{2,3}d.m and the heat accuracy functions
Matlab_Prototipes/DiffusionNd/diffusion{1,2,3}dTest.m with Laplace{1,2,3}d.m, so that the CPU
oracle's restatement of those schemes can be checked against the reference's own code without
MATLAB.

Supported: numbers, strings, identifiers, `+ - * / ^ .* ./ .^`, unary minus, comparisons,
`&&` / `||`, ranges `a:b` / `a:s:b` (a non-unit step gives a + k*s), row literals `[a b, c]`,
anonymous functions `@(w) expr`, 1-based indexing with `:` (MATLAB's outer-product semantics;
a single index is linear, column-major), indexed assignment, `function out = name(args)` and
`function [a, b] = name(args)` files, `[a, b] = f(...)`, `while` / `if` / `for` / `switch` ...
`end`, and the builtins the files call (cat, zeros, ones, size, abs, exp, sqrt, sum, max,
norm(v, inf), rem, meshgrid; plotting and printing calls are no-ops). Elementwise operations are
evaluated one at a time in the order the source writes them, as MATLAB does, so results match
MATLAB's double arithmetic operation by operation (ranges with a non-unit step may differ from
MATLAB's colon in the last bit, and exp is the C library's, which MATLAB's may differ from in
the last bit). Anything outside the subset raises an error instead of guessing.
"""
from __future__ import annotations

import math
import re
from pathlib import Path

import numpy as np

_TOKEN = re.compile(r"""
  (?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?)
| (?P<str>'(?:[^'\n]|'')*')
| (?P<id>[A-Za-z_]\w*)
| (?P<op>\.\*|\./|\.\^|==|~=|<=|>=|&&|\|\||[-+*/^()\[\],;:=<>@])
| (?P<nl>\n)
| (?P<ws>[ \t\r]+)
""", re.X)

_NOOP_CALLS = {"surf", "plot", "axis", "view", "drawnow", "shg", "title", "xlabel", "ylabel",
               "zlabel", "colorbar", "print", "figure", "hold", "grid", "fprintf", "disp", "tic",
               "toc", "clc", "clear", "close"}


class MatlabError(RuntimeError):
    pass


def _strip(src: str) -> str:
    """Removes % comments and joins `...` continuation lines, leaving strings intact. A quote
    directly after a value (MATLAB's transpose) is outside the subset."""
    out, i, n = [], 0, len(src)
    while i < n:
        c = src[i]
        if c == "%":
            while i < n and src[i] != "\n":
                i += 1
            continue
        if src.startswith("...", i):
            while i < n and src[i] != "\n":
                i += 1
            out.append(" ")
            i += 1
            continue
        if c == "'":
            before = src[i - 1] if i else ""
            if before and (before.isalnum() or before in "_)]}.'"):  # a quote right after a value
                raise MatlabError("transpose is outside the subset")
            j = i + 1
            while j < n and not (src[j] == "'" and not src.startswith("''", j)):
                if src[j] == "\n":
                    raise MatlabError("unterminated string")
                j += 2 if src.startswith("''", j) else 1
            out.append(src[i:j + 1])
            i = j + 1
            continue
        out.append(c)
        i += 1
    return "".join(out)


def _tokenize(src: str):
    """Tokens as (kind, text). Whitespace is kept only directly inside [ ] (element separator)."""
    toks, stack, pos = [], [], 0
    while pos < len(src):
        m = _TOKEN.match(src, pos)
        if not m:
            raise MatlabError(f"unexpected character {src[pos]!r}")
        pos = m.end()
        kind = m.lastgroup
        text = m.group()
        if kind == "ws":
            if stack and stack[-1] == "[":
                toks.append(("ws", " "))
            continue
        if kind == "op" and text in "([":
            stack.append(text)
        elif kind == "op" and text in ")]":
            if not stack:
                raise MatlabError("unbalanced " + text)
            stack.pop()
        toks.append((kind, text))
    toks.append(("eof", ""))
    return toks


# ---------------------------------------------------------------------------- parser (AST)
class _Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0
        self.depth_bracket = 0

    def peek(self, k=0):
        return self.t[self.i + k]

    def next(self):
        tok = self.t[self.i]
        self.i += 1
        return tok

    def accept(self, text):
        if self.peek()[1] == text and self.peek()[0] in ("op", "id"):
            self.i += 1
            return True
        return False

    def expect(self, text):
        if not self.accept(text):
            raise MatlabError(f"expected {text!r}, found {self.peek()[1]!r}")

    def skip_ws(self):
        while self.peek()[0] == "ws":
            self.i += 1

    # statements ------------------------------------------------------------------------
    def block(self, terminators):
        body = []
        while True:
            tok = self.peek()
            if tok[0] == "eof":
                if terminators:
                    raise MatlabError("missing end")
                return body
            if tok[0] == "nl" or tok[1] in (";", ","):
                self.next()
                continue
            if tok[0] == "id" and tok[1] in terminators:
                return body
            body.append(self.statement())

    def statement(self):
        tok = self.peek()
        if tok == ("id", "while"):
            self.next()
            cond = self.expr()
            body = self.block({"end"})
            self.expect("end")
            return ("while", cond, body)
        if tok == ("id", "if"):
            self.next()
            branches = [(self.expr(), self.block({"elseif", "else", "end"}))]
            orelse = []
            while True:
                if self.accept("elseif"):
                    branches.append((self.expr(), self.block({"elseif", "else", "end"})))
                elif self.accept("else"):
                    orelse = self.block({"end"})
                else:
                    self.expect("end")
                    return ("if", branches, orelse)
        if tok == ("id", "for"):
            self.next()
            var = self.next()[1]
            self.expect("=")
            rng = self.expr()
            body = self.block({"end"})
            self.expect("end")
            return ("for", var, rng, body)
        if tok == ("id", "switch"):
            self.next()
            subject = self.expr()
            cases, otherwise = [], []
            while True:
                while self.peek()[0] == "nl" or self.peek()[1] in (";", ","):
                    self.next()
                if self.accept("case"):
                    value = self.expr()
                    cases.append((value, self.block({"case", "otherwise", "end"})))
                elif self.accept("otherwise"):
                    otherwise = self.block({"case", "otherwise", "end"})
                else:
                    self.expect("end")
                    return ("switch", subject, cases, otherwise)
        # multiple assignment `[a, b] = f(...)`
        if tok == ("op", "["):
            save = self.i
            self.next()
            names = []
            while True:
                self.skip_ws()
                if self.peek()[0] != "id":
                    break
                names.append(self.next()[1])
                self.skip_ws()
                if not self.accept(","):
                    break
            if names and self.accept("]") and self.peek()[1] == "=":
                self.next()
                return ("massign", names, self.expr())
            self.i = save
        # command syntax of a no-op call (`close all`): skip to the end of the statement
        if tok[0] == "id" and tok[1] in _NOOP_CALLS and self.peek(1)[0] == "id":
            while self.peek()[0] not in ("nl", "eof") and self.peek()[1] not in (";", ","):
                self.next()
            return ("expr", ("num", 0.0))
        # assignment `name = e` / `name(args) = e`, or a bare call
        if tok[0] == "id":
            save = self.i
            name = self.next()[1]
            args = None
            if self.peek()[1] == "(":
                self.next()
                args = self.args()
            if self.peek()[1] == "=" and self.peek(1)[1] != "=":
                self.next()
                return ("assign", name, args, self.expr())
            self.i = save
        return ("expr", self.expr())

    # expressions -----------------------------------------------------------------------
    def expr(self):
        return self.oror()

    def oror(self):
        left = self.andand()
        while self.peek()[1] == "||":
            self.next()
            left = ("or", left, self.andand())
        return left

    def andand(self):
        left = self.comparison()
        while self.peek()[1] == "&&":
            self.next()
            left = ("and", left, self.comparison())
        return left

    def comparison(self):
        left = self.range_()
        while self.peek()[1] in ("<", ">", "<=", ">=", "==", "~="):
            op = self.next()[1]
            left = ("bin", op, left, self.range_())
        return left

    def range_(self):
        first = self.additive()
        if self.peek()[1] == ":" and self.depth_bracket == 0:
            self.next()
            second = self.additive()
            if self.peek()[1] == ":":
                self.next()
                return ("range", first, second, self.additive())
            return ("range", first, None, second)
        return first

    def _element_break(self):
        # inside [ ], `a -b` starts a new element; `a - b` and `a-b` do not
        return (self.depth_bracket > 0 and self.peek()[0] == "ws" and self.peek(1)[1] in ("+", "-")
                and self.peek(2)[0] != "ws")

    def additive(self):
        left = self.mult()
        while True:
            if self._element_break():
                return left
            save = self.i
            if self.depth_bracket:
                self.skip_ws()
            if self.peek()[1] in ("+", "-"):
                op = self.next()[1]
                if self.depth_bracket:
                    self.skip_ws()
                left = ("bin", op, left, self.mult())
            else:
                self.i = save
                return left

    def mult(self):
        left = self.unary()
        while True:
            save = self.i
            if self.depth_bracket:
                self.skip_ws()
            if self.peek()[1] in ("*", "/", ".*", "./"):
                op = self.next()[1]
                if self.depth_bracket:
                    self.skip_ws()
                left = ("bin", op, left, self.unary())
            else:
                self.i = save
                return left

    def unary(self):
        if self.peek()[1] in ("-", "+"):
            op = self.next()[1]
            operand = self.unary()
            return ("neg", operand) if op == "-" else operand
        return self.power()

    def power(self):
        left = self.postfix()
        while self.peek()[1] in ("^", ".^"):
            op = self.next()[1]
            if self.peek()[1] in ("-", "+"):
                sign = self.next()[1]
                rhs = self.postfix()
                rhs = ("neg", rhs) if sign == "-" else rhs
            else:
                rhs = self.postfix()
            left = ("bin", op, left, rhs)
        return left

    def postfix(self):
        node = self.primary()
        while self.peek()[1] == "(":
            self.next()
            node = ("call", node, self.args())
        return node

    def args(self):
        out = []
        saved = self.depth_bracket
        self.depth_bracket = 0
        if self.accept(")"):
            self.depth_bracket = saved
            return out
        while True:
            if self.peek()[1] == ":" and self.peek(1)[1] in (",", ")"):
                self.next()
                out.append(("colon",))
            else:
                out.append(self.expr())
            if self.accept(")"):
                break
            self.expect(",")
        self.depth_bracket = saved
        return out

    def primary(self):
        kind, text = self.next()
        if kind == "num":
            return ("num", float(text))
        if kind == "str":
            return ("str", text[1:-1].replace("''", "'"))
        if kind == "id":
            return ("id", text)
        if text == "(":
            saved = self.depth_bracket
            self.depth_bracket = 0
            e = self.expr()
            self.depth_bracket = saved
            self.expect(")")
            return e
        if text == "[":
            self.depth_bracket += 1
            elems = []
            self.skip_ws()
            while not self.accept("]"):
                elems.append(self.expr())
                self.skip_ws()
                self.accept(",")
                self.skip_ws()
            self.depth_bracket -= 1
            return ("row", elems)
        if text == "@":
            self.expect("(")
            params = []
            while not self.accept(")"):
                params.append(self.next()[1])
                self.accept(",")
            return ("lambda", params, self.expr())
        raise MatlabError(f"unexpected token {text!r}")


# ---------------------------------------------------------------------------- evaluation
def _is_scalar(v) -> bool:
    return np.ndim(v) == 0 or np.size(v) == 1


def _scalar(v) -> float:
    return float(np.asarray(v).reshape(-1)[0])


def _as_index(v, extent):
    if isinstance(v, tuple) and v == ("colon",):
        return np.arange(extent)
    a = np.asarray(v, dtype=np.float64).reshape(-1)
    if np.any(a != np.round(a)) or np.any(a < 1):
        raise MatlabError("non-integer or non-positive index")
    return a.astype(np.int64) - 1


def _squeeze_trailing(a):
    while a.ndim > 2 and a.shape[-1] == 1:
        a = a[..., 0]
    return a


def _scalar_index(shape, idx):
    """Zero-based multi-index of all-scalar MATLAB indices (a single one is linear,
    column-major), or None when any index is not a scalar."""
    if not all(isinstance(v, (float, int)) for v in idx):
        return None
    ints = [int(v) for v in idx]
    if any(v != w or v < 1 for v, w in zip(ints, idx)):
        raise MatlabError("non-integer or non-positive index")
    if len(ints) == 1:
        if ints[0] > int(np.prod(shape)):
            raise MatlabError("index out of range")
        return np.unravel_index(ints[0] - 1, shape, order="F")
    if len(ints) < len(shape) or any(v != 1 for v in ints[len(shape):]):
        return None
    out = tuple(v - 1 for v in ints[:len(shape)])
    if any(v >= n for v, n in zip(out, shape)):
        raise MatlabError("index out of range")
    return out


def _index(arr, idx):
    arr = np.asarray(arr, dtype=np.float64)
    if arr.ndim < 2:
        arr = arr.reshape(1, -1)
    at = _scalar_index(arr.shape, idx)
    if at is not None:
        return float(arr[at])
    if len(idx) == 1:
        flat = arr.reshape(-1, order="F")
        if isinstance(idx[0], tuple):
            return flat.reshape(-1, 1).copy()
        sel = _as_index(idx[0], flat.size)
        out = flat[sel]
        return out.reshape(1, -1) if arr.shape[0] == 1 else out.reshape(-1, 1)
    if len(idx) < arr.ndim:
        raise MatlabError("fewer indices than dimensions is outside the subset")
    view = arr.reshape(arr.shape + (1,) * (len(idx) - arr.ndim))
    sel = [_as_index(v, view.shape[d]) for d, v in enumerate(idx)]
    return _squeeze_trailing(view[np.ix_(*sel)].copy())


def _matlab_max(a):
    a = np.asarray(a, dtype=np.float64)
    if a.ndim < 2 or min(a.shape[:2]) == 1 and a.ndim == 2:
        return float(np.max(a))
    raise MatlabError("max over a matrix is outside the subset")


def _cat(dim, *arrays):
    d = int(dim) - 1
    mats = []
    for a in arrays:
        a = np.asarray(a, dtype=np.float64)
        if a.ndim < 2:
            a = a.reshape(1, -1)
        while a.ndim <= d:
            a = a[..., None]
        mats.append(a)
    nd = max(m.ndim for m in mats)
    mats = [m.reshape(m.shape + (1,) * (nd - m.ndim)) for m in mats]
    return _squeeze_trailing(np.concatenate(mats, axis=d))


def _zeros(*args):
    if len(args) == 1:
        shape = tuple(int(x) for x in np.asarray(args[0]).reshape(-1))
        if len(shape) == 1:
            shape = (shape[0], shape[0])
    else:
        shape = tuple(int(_scalar(x)) for x in args)
    return np.zeros(shape)


def _ones(*args):
    return _zeros(*args) + 1.0


def _elementwise(fn, a):
    """A C-library elementary function applied value by value (numpy's vectorised versions may
    round differently from the C library the oracle calls)."""
    if isinstance(a, float):
        return fn(a)
    arr = np.asarray(a, dtype=np.float64)
    return np.array([fn(float(v)) for v in arr.reshape(-1)], dtype=np.float64).reshape(arr.shape)


def _matlab_sum(a):
    a = np.asarray(a, dtype=np.float64)
    if a.ndim <= 2 and (a.ndim < 2 or min(a.shape) == 1):
        total = 0.0
        for v in a.reshape(-1):  # left to right, one rounding per addition
            total += float(v)
        return total
    raise MatlabError("sum over a matrix is outside the subset")


def _matlab_min(a):
    a = np.asarray(a, dtype=np.float64)
    if a.ndim < 2 or min(a.shape[:2]) == 1 and a.ndim == 2:
        return float(np.min(a))
    raise MatlabError("min over a matrix is outside the subset")


def _rectangular_pulse(a, b, x):
    """MATLAB's rectangularPulse(a, b, x) for a < b: 1 inside (a, b), 1/2 at x = a or b, else 0."""
    a, b = _scalar(a), _scalar(b)
    if not a < b:
        raise MatlabError("rectangularPulse with a >= b is outside the subset")
    x = np.asarray(x, dtype=np.float64)
    return np.where((x > a) & (x < b), 1.0, np.where((x == a) | (x == b), 0.5, 0.0))


def _norm(a, p=2.0):
    a = np.asarray(a, dtype=np.float64)
    if (a.ndim < 2 or min(a.shape) == 1) and np.isinf(p):
        return float(np.max(np.abs(a)))
    raise MatlabError("only the vector infinity norm is in the subset")


def _meshgrid(*axes):
    vs = [np.asarray(v, dtype=np.float64).reshape(-1) for v in axes]
    if len(vs) == 2:
        x, y = np.meshgrid(vs[0], vs[1], indexing="xy")
        return x, y
    if len(vs) == 3:
        x, y, z = np.meshgrid(vs[0], vs[1], vs[2], indexing="xy")  # (ny, nx, nz), as MATLAB
        return x, y, z
    raise MatlabError("meshgrid of 2 or 3 vectors only")


BUILTINS = {
    "cat": _cat,
    "zeros": _zeros,
    "ones": _ones,
    "size": lambda a: np.array(np.shape(a) if np.ndim(a) >= 2 else (1, np.size(a)),
                               dtype=np.float64).reshape(1, -1),
    "abs": lambda a: np.abs(np.asarray(a, dtype=np.float64)),
    "exp": lambda a: _elementwise(math.exp, a),
    "max": _matlab_max,
    "min": _matlab_min,
    "rectangularPulse": _rectangular_pulse,
    "rem": lambda a, b: float(np.fmod(_scalar(a), _scalar(b))),
    "sqrt": lambda a: np.sqrt(a) if isinstance(a, float) else np.sqrt(np.asarray(a, dtype=np.float64)),
    "sum": _matlab_sum,
    "norm": _norm,
    "meshgrid": _meshgrid,
    "inf": lambda: np.inf,
    "Inf": lambda: np.inf,
    "pi": lambda: np.pi,
}
_MULTI_OUTPUT = {"meshgrid"}


class Interpreter:
    """Runs statements of the subset; functions not in the environment are loaded from
    `<name>.m` in `fdir`."""

    def __init__(self, fdir: Path | None = None):
        self.fdir = Path(fdir) if fdir else None
        self._files: dict[str, tuple] = {}
        self.calls: dict[str, int] = {}
        self._end: list[float] = []  # the value of `end` inside the index being evaluated

    # -- entry points -------------------------------------------------------------------
    def run(self, src: str, env: dict) -> dict:
        body = _Parser(_tokenize(_strip(src))).block(set())
        self._exec(body, env)
        return env

    def call_file(self, name: str, args: list, nargout: int = 1, env_out: dict | None = None):
        """Runs function file `name`.m; returns its first output, or a list of the first
        `nargout` outputs. env_out, if given, receives the function's final workspace."""
        if name not in self._files:
            if self.fdir is None:
                raise MatlabError(f"unknown function {name}")
            src = _strip((self.fdir / f"{name}.m").read_text())
            m = re.match(r"\s*function\s+(?:\[([^\]]*)\]|(\w+))\s*=\s*(\w+)\s*\(([^)]*)\)", src)
            if not m or m.group(3) != name:
                raise MatlabError(f"{name}.m is not a function file")
            outs = [o.strip() for o in (m.group(1) or m.group(2)).split(",") if o.strip()]
            params = [p.strip() for p in m.group(4).split(",") if p.strip()]
            body = _Parser(_tokenize(src[m.end():])).block(set())
            self._files[name] = (outs, params, body)
        outs, params, body = self._files[name]
        if len(args) != len(params):
            raise MatlabError(f"{name} takes {len(params)} arguments")
        if nargout > len(outs):
            raise MatlabError(f"{name} has {len(outs)} outputs")
        self.calls[name] = self.calls.get(name, 0) + 1
        env = dict(zip(params, args))
        self._exec(body, env)
        if env_out is not None:
            env_out.update(env)
        return env[outs[0]] if nargout == 1 else [env[o] for o in outs[:nargout]]

    # -- statements ---------------------------------------------------------------------
    def _exec(self, body, env):
        for st in body:
            kind = st[0]
            if kind == "assign":
                _, name, args, e = st
                val = self._eval(e, env)
                if args is None:
                    env[name] = val
                else:
                    self._assign_index(env, name, args, val)
            elif kind == "expr":
                self._eval(st[1], env)
            elif kind == "while":
                guard = 0
                while self._truth(self._eval(st[1], env)):
                    self._exec(st[2], env)
                    guard += 1
                    if guard > 1_000_000:
                        raise MatlabError("while loop did not end")
            elif kind == "if":
                for cond, body in st[1]:
                    if self._truth(self._eval(cond, env)):
                        self._exec(body, env)
                        break
                else:
                    self._exec(st[2], env)
            elif kind == "for":
                rng = np.asarray(self._eval(st[2], env), dtype=np.float64).reshape(-1)
                for v in rng:
                    env[st[1]] = float(v)
                    self._exec(st[3], env)
            elif kind == "switch":
                subject = self._eval(st[1], env)
                for value, body in st[2]:
                    v = self._eval(value, env)
                    same = (subject == v) if isinstance(subject, str) or isinstance(v, str) else \
                        bool(np.all(np.asarray(subject) == np.asarray(v)))
                    if same:
                        self._exec(body, env)
                        break
                else:
                    self._exec(st[3], env)
            elif kind == "massign":
                names, e = st[1], st[2]
                if e[0] != "call" or e[1][0] != "id":
                    raise MatlabError("multiple assignment needs a function call")
                vals = self._eval(e, env, nargout=len(names))
                for nm, v in zip(names, vals):
                    env[nm] = v
            else:
                raise MatlabError("statement kind " + kind)

    @staticmethod
    def _truth(v) -> bool:
        a = np.asarray(v)
        return bool(a.size) and bool(np.all(a != 0))

    def _assign_index(self, env, name, args, val):
        arr = env[name]
        if not isinstance(arr, np.ndarray):
            raise MatlabError("indexed assignment to a non-array")
        idx = [("colon",) if a == ("colon",) else self._eval(a, env) for a in args]
        at = _scalar_index(arr.shape, idx)
        if at is not None:
            if not _is_scalar(val):
                raise MatlabError("assignment of an array to one element")
            arr[at] = _scalar(val)
            return
        if len(idx) == 1:  # linear (column-major) positions
            flat = _as_index(idx[0], arr.size)
            pos = np.unravel_index(flat, arr.shape, order="F")
            v = np.asarray(val, dtype=np.float64).reshape(-1)
            if v.size not in (1, flat.size):
                raise MatlabError("linear assignment of a wrong number of values")
            arr[pos] = v
            return
        if len(idx) < arr.ndim:
            raise MatlabError("fewer indices than dimensions is outside the subset")
        view = arr.reshape(arr.shape + (1,) * (len(idx) - arr.ndim))
        if not np.shares_memory(view, arr):
            raise MatlabError("indexed assignment needs a contiguous array")
        sel = [_as_index(v, view.shape[d]) for d, v in enumerate(idx)]
        target_shape = tuple(len(s) for s in sel)
        v = np.asarray(val, dtype=np.float64)
        if v.size != 1:
            v = v.reshape(v.shape + (1,) * (len(target_shape) - v.ndim))
            if v.shape != target_shape:
                raise MatlabError(f"assignment shape {v.shape} into {target_shape}")
        view[np.ix_(*sel)] = v

    # -- expressions --------------------------------------------------------------------
    def _eval(self, n, env, nargout: int = 1):
        kind = n[0]
        if kind == "num":
            return n[1]
        if kind == "str":
            return n[1]
        if kind == "and":
            return 1.0 if self._truth(self._eval(n[1], env)) and self._truth(self._eval(n[2], env)) else 0.0
        if kind == "or":
            return 1.0 if self._truth(self._eval(n[1], env)) or self._truth(self._eval(n[2], env)) else 0.0
        if kind == "id":
            name = n[1]
            if name in env:
                return env[name]
            if name == "end":
                if not self._end:
                    raise MatlabError("`end` outside an index")
                return self._end[-1]
            if name in _NOOP_CALLS:
                return None
            if name in BUILTINS:
                return BUILTINS[name]()
            return self.call_file(name, [])
        if kind == "neg":
            return -self._eval(n[1], env)
        if kind == "bin":
            return self._binary(n[1], self._eval(n[2], env), self._eval(n[3], env))
        if kind == "range":
            a = _scalar(self._eval(n[1], env))
            s = 1.0 if n[2] is None else _scalar(self._eval(n[2], env))
            b = _scalar(self._eval(n[3], env))
            if s == 0.0:
                raise MatlabError("range with a zero step")
            q = (b - a) / s
            k = round(q) if abs(q - round(q)) <= 1e-10 * max(1.0, abs(q)) else math.floor(q)
            return (a + s * np.arange(max(int(k) + 1, 0), dtype=np.float64)).reshape(1, -1)
        if kind == "row":
            vals = [self._eval(e, env) for e in n[1]]
            if all(_is_scalar(v) for v in vals):
                return np.array([_scalar(v) for v in vals], dtype=np.float64).reshape(1, -1)
            return _cat(2, *vals)
        if kind == "lambda":
            params, body = n[1], n[2]
            closure = dict(env)

            def fn(*args):
                local = dict(closure)
                local.update(zip(params, args))
                return self._eval(body, local)
            return fn
        if kind == "call":
            target = n[1]
            if target[0] == "id":
                name = target[1]
                if name in env and isinstance(env[name], (np.ndarray, float)):
                    arr = env[name]
                    shape = np.shape(arr) if np.ndim(arr) >= 2 else (1, int(np.size(arr)))
                    idx = []
                    for d, a in enumerate(n[2]):
                        if a == ("colon",):
                            idx.append(a)
                            continue
                        extent = int(np.prod(shape)) if len(n[2]) == 1 else (shape[d] if d < len(shape) else 1)
                        self._end.append(float(extent))
                        try:
                            idx.append(self._eval(a, env))
                        finally:
                            self._end.pop()
                    return _index(arr, idx)
                if name not in env and name in _NOOP_CALLS:
                    return None  # plotting: its arguments are never evaluated
                args = [self._eval(a, env) for a in n[2]]
                if name in env and callable(env[name]):
                    return env[name](*args)
                if name in BUILTINS:
                    out = BUILTINS[name](*args)
                    if name in _MULTI_OUTPUT:
                        return list(out[:nargout]) if nargout > 1 else out[0]
                    if nargout > 1:
                        raise MatlabError(f"{name} has one output")
                    return out
                return self.call_file(name, args, nargout)
            raise MatlabError("call of an expression")
        raise MatlabError("node kind " + kind)

    @staticmethod
    def _binary(op, a, b):
        fa = np.asarray(a, dtype=np.float64) if not isinstance(a, float) else a
        fb = np.asarray(b, dtype=np.float64) if not isinstance(b, float) else b
        if op in ("+", "-", ".*", "./", ".^", "<", ">", "<=", ">=", "==", "~="):
            if op == "+":
                return fa + fb
            if op == "-":
                return fa - fb
            if op == ".*":
                return fa * fb
            if op == "./":
                return fa / fb
            if op == ".^":
                return np.power(fa, fb)
            r = {"<": np.less, ">": np.greater, "<=": np.less_equal, ">=": np.greater_equal,
                 "==": np.equal, "~=": np.not_equal}[op](fa, fb)
            return np.asarray(r, dtype=np.float64)
        if op == "*":
            if _is_scalar(fa) or _is_scalar(fb):
                return fa * fb
            raise MatlabError("matrix product is outside the subset")
        if op == "/":
            if _is_scalar(fb):
                return fa / fb
            raise MatlabError("matrix division is outside the subset")
        if op == "^":
            if _is_scalar(fa) and _is_scalar(fb):
                return np.power(fa, fb)
            raise MatlabError("matrix power is outside the subset")
        raise MatlabError("operator " + op)
