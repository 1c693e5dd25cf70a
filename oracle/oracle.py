"""Python handle on the CPU oracle (advdiff_oracle.cpp) -- TEST INFRASTRUCTURE ONLY.

The oracle restates the reference's schemes in FP64 (and FP32 for error-floor studies). Only the
tests, the smoke check and the benchmark's CPU-baseline leg use it; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SO = HERE / "_build" / "liboracle.so"
SRC = HERE / "advdiff_oracle.cpp"
SOURCES = [SRC, HERE / "cpu_baseline.cpp"]

_lib = None
_D, _I, _I64, _U32 = C.c_double, C.c_int, C.c_int64, C.c_uint32
_PD = C.POINTER(C.c_double)
_HEAT = [_I, _I, _I, _I, _I, _I, _I, _I, _D, _D, _D, _D]
_BURG = [_I, _I, _I, _I, _I, _I, _I, _D, _D, _D, _D, _D, _D]


def build() -> Path:
    """Compiles liboracle.so with g++ (the same flags as oracle/Makefile)."""
    if not SO.exists() or any(SO.stat().st_mtime < s.stat().st_mtime for s in SOURCES):
        SO.parent.mkdir(parents=True, exist_ok=True)
        cxx = os.environ.get("CXX", "g++")
        subprocess.run([cxx, "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                        "-o", str(SO), *map(str, SOURCES)], check=True)
    return SO


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(SO))
        sig = {
            "orc_heat_stage_f64": (None, _HEAT + [_I, C.c_void_p, C.c_void_p, C.c_void_p]),
            "orc_heat_stage_f32": (None, _HEAT + [_I, C.c_void_p, C.c_void_p, C.c_void_p]),
            "orc_heat_run_f64": (None, _HEAT + [_I, _I64, C.c_void_p]),
            "orc_heat_run_f32": (None, _HEAT + [_I, _I64, C.c_void_p]),
            "orc_heat_stage_f32_fma": (None, _HEAT + [_I, C.c_void_p, C.c_void_p, C.c_void_p]),
            "orc_heat_run_f32_fma": (None, _HEAT + [_I, _I64, C.c_void_p]),
            "orc_heat_stage_f64_fma": (None, _HEAT + [_I, C.c_void_p, C.c_void_p, C.c_void_p]),
            "orc_heat_run_f64_fma": (None, _HEAT + [_I, _I64, C.c_void_p]),
            "orc_heat_ref_constants": (None, [_I, _D, _I, _I, _I, _I, _I, _I, _I] + [_PD] * 8),
            "orc_ic_heat_ref": (None, [_I, _I, _I, _I, _D, _D, _D, C.c_void_p]),
            "orc_heat_accuracy": (_I, [_I, _I, _D, _D, _PD, _PD, _PD]),
            "orc_ic_heat2d_gauss_noise": (None, [_I, _I, _U32, _D, C.c_void_p]),
            "orc_heat3d_blob_params": (None, [_U32, _I, C.c_void_p]),
            "orc_ic_heat3d_blobs": (None, [_I, _I, _I, _U32, _I, C.c_void_p]),
            "orc_burgers_fourier_params": (None, [_U32, _I, _D, C.c_void_p]),
            "orc_ic_burgers_fourier": (None, [_I, _I, _I, _D, _U32, _I, _D, C.c_void_p]),
            "orc_ic_burgers_ref": (None, [_I, _I, _I, _D, _D, _D, C.c_void_p]),
            "orc_burgers_rhs_f64": (None, _BURG + [C.c_void_p, _D, C.c_void_p]),
            "orc_burgers_rhs_f32": (None, _BURG + [_I, C.c_void_p, C.c_float, C.c_void_p]),
            "orc_burgers_stage_f64": (None, _BURG + [_I, C.c_void_p, C.c_void_p, _D, C.c_void_p, C.c_void_p]),
            "orc_burgers_stage_f32": (None, _BURG + [_I, _I, C.c_void_p, C.c_void_p, _D, C.c_void_p, C.c_void_p]),
            "orc_burgers_run_f64": (_I64, _BURG + [C.c_void_p, _D, _D, _I, _D, _I64, _PD]),
            "orc_burgers_run_f32": (_I64, _BURG + [_I, C.c_void_p, _D, _D, _I, _D, _I64, _PD]),
            "orc_burgers_ref_steps": (_I64, [_D, _D, _D, _D, _D, _I, _I, _I, _D, _PD]),
            "orc_burgers_run_recip_f64": (_I64, _BURG + [C.c_void_p, _D, _D, _I, _D, _I64, _PD]),
            "orc_burgers_sweep_all_f64": (None, [_I, _I, _I, _I, _I, _D, C.c_void_p, C.c_void_p]),
            "orc_burgers_sweep_all_f32": (None, [_I, _I, _I, _I, _I, _D, C.c_void_p, C.c_void_p]),
            "orc_heat_blocking_run_f64": (None, [_I, _I, _I, _D, _D, _D, _D, _I64, C.c_void_p]),
            "orc_max_abs_f64": (_D, [C.c_void_p, _I64]),
            "orc_burgers_step_adjoint_f64": (None, _BURG + [C.c_void_p] * 3 + [_D, C.c_void_p]),
            "orc_burgers_step_adjoint_f32": (None, _BURG + [C.c_void_p] * 3 + [_D, C.c_void_p]),
            "orc_heatk_step_f64": (None, [_I, _I, _I, _I, _D, _D, _D] + [C.c_void_p] * 3),
            "orc_heatk_step_f32": (None, [_I, _I, _I, _I, _D, _D, _D] + [C.c_void_p] * 3),
            "orc_heatk_adjoint_f64": (None, [_I, _I, _I, _I, _D, _D, _D] + [C.c_void_p] * 5),
            "orc_heatk_adjoint_f32": (None, [_I, _I, _I, _I, _D, _D, _D] + [C.c_void_p] * 5),
            "orc_philox_u01x2": (None, [_U32, _U32, C.c_uint64, _PD, _PD]),
            "orc_proto_residual_f64": (None, [_I, _I, _I, _I, _I, _I, _D, C.c_void_p, C.c_void_p]),
            "orc_proto_run_f64": (_I64, [_I, _I, _I, _I, _I, _PD, _D, _D, _I64, C.c_void_p, _PD]),
            "orc_weno7_side_f64": (_D, [_PD]),
            "orc_lsrk54_gain": (None, [_D, _D, _PD, _PD]),
            "orc_cpu_heat_euler_o2_f32": (None, [_I, _I, _I, _I, _I, _I, _D, _D, _D, _D, _I64, C.c_void_p,
                                                  C.c_void_p]),
            "orc_num_threads": (_I, []),
            "orc_set_num_threads": (None, [_I]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray) -> int:
    assert a.flags.c_contiguous
    return a.ctypes.data


def _heat_args(ndim, nx, ny, nz, order, frozen, zero_boundary, periodic, kx, ky, kz, dt):
    return [ndim, nx, ny, nz if ndim == 3 else 1, order, frozen, int(zero_boundary), int(periodic), kx, ky, kz, dt]


def heat_stage(cfg, stage: int, uin: np.ndarray, un: np.ndarray, periodic: bool = False,
               fp32_order: str = "gpu") -> np.ndarray:
    """One stage with the scheme of a solvers.HeatConfig-like object (ndim, nx.., order, ...).
    FP32 inputs use the GPU path's fused-multiply-add order unless fp32_order == "reference"; FP64
    inputs use it when the configuration asks for the contracted form (cfg.contract)."""
    out = np.empty_like(uin)
    if uin.dtype == np.float64:
        f = lib().orc_heat_stage_f64_fma if getattr(cfg, "contract", False) else lib().orc_heat_stage_f64
    else:
        f = lib().orc_heat_stage_f32 if fp32_order == "reference" else lib().orc_heat_stage_f32_fma
    f(*_heat_args(cfg.ndim, cfg.nx, cfg.ny, cfg.nz, cfg.order, cfg.frozen, cfg.zero_boundary, periodic,
                  cfg.kx, cfg.ky, cfg.kz, cfg.dt), stage, _p(uin), _p(un), _p(out))
    return out


def heat_run(cfg, u: np.ndarray, nsteps: int, time: int, fp32_order: str = "gpu") -> np.ndarray:
    u = np.ascontiguousarray(u).copy()
    if u.dtype == np.float64:
        f = lib().orc_heat_run_f64_fma if getattr(cfg, "contract", False) else lib().orc_heat_run_f64
    else:
        f = lib().orc_heat_run_f32 if fp32_order == "reference" else lib().orc_heat_run_f32_fma
    f(*_heat_args(cfg.ndim, cfg.nx, cfg.ny, cfg.nz, cfg.order, cfg.frozen, cfg.zero_boundary, False,
                  cfg.kx, cfg.ky, cfg.kz, cfg.dt), time, nsteps, _p(u))
    return u


def cpu_heat_euler_o2(cfg, u: np.ndarray, nsteps: int, work: np.ndarray | None = None) -> np.ndarray:
    """nsteps forward-Euler O2 steps of an FP32 state with the tuned CPU loop of the benchmark's
    CPU baseline (cpu_baseline.cpp); in place on u, which is returned. Equal bit for bit to
    heat_run(cfg, u, nsteps, 0, fp32_order="reference")."""
    assert u.dtype == np.float32 and u.flags.c_contiguous and cfg.order == 2
    if work is None:
        work = np.empty_like(u)
    lib().orc_cpu_heat_euler_o2_f32(cfg.ndim, cfg.nx, cfg.ny, cfg.nz if cfg.ndim == 3 else 1, cfg.frozen,
                                    int(cfg.zero_boundary), cfg.kx, cfg.ky, cfg.kz, cfg.dt, nsteps, _p(u), _p(work))
    return u


def heat_accuracy(dim: int, nc: int, tEnd: float, factor: float):
    L1, L2, Li = C.c_double(), C.c_double(), C.c_double()
    it = lib().orc_heat_accuracy(dim, nc, tEnd, factor, C.byref(L1), C.byref(L2), C.byref(Li))
    return it, L1.value, L2.value, Li.value


def heat_ref_constants(ndim, Cc, L, W, H, nx, ny, nz, iters):
    out = [C.c_double() for _ in range(8)]
    lib().orc_heat_ref_constants(ndim, Cc, L, W, H, nx, ny, nz, iters, *[C.byref(o) for o in out])
    return dict(zip(["dx", "dy", "dz", "dt", "kx", "ky", "kz", "tFinal"], [o.value for o in out]))


def ic_heat_ref(ndim, nx, ny, nz, dx, dy, dz) -> np.ndarray:
    u = np.empty(nx * ny * (nz if ndim == 3 else 1))
    lib().orc_ic_heat_ref(ndim, nx, ny, nz, dx, dy, dz, _p(u))
    return u


def ic_heat2d_gauss_noise(nx, ny, seed, sigma) -> np.ndarray:
    u = np.empty(nx * ny)
    lib().orc_ic_heat2d_gauss_noise(nx, ny, seed, sigma, _p(u))
    return u


def ic_heat3d_blobs(nx, ny, nz, seed, nblobs=8) -> np.ndarray:
    u = np.empty(nx * ny * nz)
    lib().orc_ic_heat3d_blobs(nx, ny, nz, seed, nblobs, _p(u))
    return u


def heat3d_blob_params(seed, nblobs=8) -> np.ndarray:
    p = np.empty(4 * nblobs)
    lib().orc_heat3d_blob_params(seed, nblobs, _p(p))
    return p.reshape(nblobs, 4)


def burgers_fourier_params(seed, nmodes=16, amax=0.1) -> np.ndarray:
    p = np.empty(5 * nmodes)
    lib().orc_burgers_fourier_params(seed, nmodes, amax, _p(p))
    return p.reshape(nmodes, 5)


def ic_burgers_fourier(nx, ny, nz, L, seed, nmodes=16, amax=0.1) -> np.ndarray:
    u = np.empty(nx * ny * nz)
    lib().orc_ic_burgers_fourier(nx, ny, nz, L, seed, nmodes, amax, _p(u))
    return u


def ic_burgers_ref(nx, ny, nz, dx, dy, dz) -> np.ndarray:
    u = np.empty(nx * ny * nz)
    lib().orc_ic_burgers_ref(nx, ny, nz, dx, dy, dz, _p(u))
    return u


def _burg_args(cfg):
    k = [cfg.C / (12 * h * h) if cfg.C else 0.0 for h in (cfg.dx, cfg.dy, cfg.dz)]
    if cfg.nz == 1:  # 2D: no z term
        k[2] = 0.0
    return [cfg.nx, cfg.ny, cfg.nz, int(cfg.weno == 1), int(cfg.lf == 1), int(cfg.bc == 1), int(cfg.bug_b2),
            cfg.dx, cfg.dy, cfg.dz, *k]


def burgers_stage(cfg, stage, uin, un, dt, div64=True):
    """One SSP-RK3 stage with the scheme of a solvers.BurgersConfig-like object."""
    out = np.empty_like(uin)
    Lu = np.zeros_like(uin)
    if uin.dtype == np.float64:
        lib().orc_burgers_stage_f64(*_burg_args(cfg), stage, _p(uin), _p(un), dt, _p(out), _p(Lu))
    else:
        lib().orc_burgers_stage_f32(*_burg_args(cfg), int(div64), stage, _p(uin), _p(un), dt, _p(out), _p(Lu))
    return out


def burgers_rhs(cfg, u, alpha):
    Lu = np.zeros_like(u)
    if u.dtype == np.float64:
        lib().orc_burgers_rhs_f64(*_burg_args(cfg), _p(u), alpha, _p(Lu))
    else:
        lib().orc_burgers_rhs_f32(*_burg_args(cfg), 1, _p(u), alpha, _p(Lu))
    return Lu


def burgers_run(cfg, u, tEnd, cfl, dt_rule, C_visc=0.0, max_steps=1 << 40, div64=True, recip=False):
    """recip: the shared-memory reference program's weight normalisation (FP64 only)."""
    u = np.ascontiguousarray(u).copy()
    t = C.c_double()
    if recip:
        assert u.dtype == np.float64
        it = lib().orc_burgers_run_recip_f64(*_burg_args(cfg), _p(u), tEnd, cfl, dt_rule, C_visc, max_steps,
                                             C.byref(t))
    elif u.dtype == np.float64:
        it = lib().orc_burgers_run_f64(*_burg_args(cfg), _p(u), tEnd, cfl, dt_rule, C_visc, max_steps, C.byref(t))
    else:
        it = lib().orc_burgers_run_f32(*_burg_args(cfg), int(div64), _p(u), tEnd, cfl, dt_rule, C_visc, max_steps,
                                       C.byref(t))
    return u, t.value, it


def burgers_sweep_all(axis: int, weno_z: bool, u: np.ndarray, h: float, Lu: np.ndarray) -> np.ndarray:
    """The shared-memory reference program's sweep along `axis` on a (nz, ny, nx) array: returns
    Lu after it (x assigns, y and z subtract; Lu is not modified in place)."""
    u = np.ascontiguousarray(u)
    out = np.ascontiguousarray(Lu).copy()
    nz, ny, nx = u.shape
    f = lib().orc_burgers_sweep_all_f64 if u.dtype == np.float64 else lib().orc_burgers_sweep_all_f32
    f(axis, int(weno_z), nx, ny, nz, h, _p(u), _p(out))
    return out


def heat_blocking_run(nx, ny, nz, kx, ky, kz, dt, iters, u: np.ndarray) -> np.ndarray:
    """The z-blocked reference heat program's loop (FP64), iters time steps from u."""
    u = np.ascontiguousarray(u, dtype=np.float64).copy()
    lib().orc_heat_blocking_run_f64(nx, ny, nz, kx, ky, kz, dt, iters, _p(u))
    return u


def burgers_ref_steps(tEnd, cfl, L, W, H, nx, ny, nz, Cv=1e-5):
    t = C.c_double()
    it = lib().orc_burgers_ref_steps(tEnd, cfl, L, W, H, nx, ny, nz, Cv, C.byref(t))
    return it, t.value


def set_threads(n: int) -> None:
    lib().orc_set_num_threads(n)


def num_threads() -> int:
    return lib().orc_num_threads()


# ------------------------------------------------------------- heat with a diffusivity field k(x)
def heatk_step(shape, zero_boundary: bool, c, k: np.ndarray, u: np.ndarray) -> np.ndarray:
    """One forward-Euler step of u_t = div(k grad u) (conservative, face averages); c = dt/h^2 per axis."""
    nx, ny, nz = shape
    out = np.empty_like(u)
    f = lib().orc_heatk_step_f64 if u.dtype == np.float64 else lib().orc_heatk_step_f32
    f(nx, ny, nz, int(zero_boundary), *c, _p(k), _p(u), _p(out))
    return out


def heatk_adjoint(shape, zero_boundary: bool, c, k, u, lam, grad):
    """Adjoint of one step: returns dJ/du^n from lam = dJ/du^{n+1}; adds the step's dJ/dk to grad."""
    nx, ny, nz = shape
    out = np.empty_like(lam)
    f = lib().orc_heatk_adjoint_f64 if u.dtype == np.float64 else lib().orc_heatk_adjoint_f32
    f(nx, ny, nz, int(zero_boundary), *c, _p(k), _p(u), _p(lam), _p(out), _p(grad))
    return out


def heatk_loss_and_gradient(shape, zero_boundary, c, k, u0, target, nsteps):
    """J = 1/2 |u(T) - target|^2 and (dJ/dk, dJ/du0) by storing every state (small cases only)."""
    states = [u0]
    for _ in range(nsteps):
        states.append(heatk_step(shape, zero_boundary, c, k, states[-1]))
    r = states[-1] - target
    J = 0.5 * float(np.dot(r.astype(np.float64), r.astype(np.float64)))
    lam = r.copy()
    grad = np.zeros_like(k)
    for n in range(nsteps - 1, -1, -1):
        lam = heatk_adjoint(shape, zero_boundary, c, k, states[n], lam, grad)
    return J, grad, lam


# ------------------------------------------------------------------- Burgers discrete adjoint
def burgers_step_adjoint(cfg, un, u1, u2, dt, lam):
    """dJ/du^n from lam = dJ/du^{n+1} and the step's stage inputs (periodic, local LF)."""
    lam = np.ascontiguousarray(lam).copy()
    f = lib().orc_burgers_step_adjoint_f64 if un.dtype == np.float64 else lib().orc_burgers_step_adjoint_f32
    f(*_burg_args(cfg), _p(un), _p(u1), _p(u2), dt, _p(lam))
    return lam


def burgers_forward_states(cfg, u0, dt, nsteps, div64=True):
    """Every stage input of nsteps fixed-dt SSP-RK3 steps: [(u^n, u1, u2)] and u^N."""
    states = []
    u = u0
    for _ in range(nsteps):
        u1 = burgers_stage(cfg, 1, u, u, dt, div64)
        u2 = burgers_stage(cfg, 2, u1, u, dt, div64)
        un1 = burgers_stage(cfg, 3, u2, u, dt, div64)
        states.append((u, u1, u2))
        u = un1
    return states, u


def burgers_loss_and_gradient(cfg, u0, target, dt, nsteps):
    """J = 1/2 |u(T) - target|^2 and dJ/du0 by storing every stage (small cases only)."""
    states, uT = burgers_forward_states(cfg, u0, dt, nsteps)
    r = uT - target
    J = 0.5 * float(np.dot(r.astype(np.float64), r.astype(np.float64)))
    lam = r.copy()
    for un, u1, u2 in reversed(states):
        lam = burgers_step_adjoint(cfg, un, u1, u2, dt, lam)
    return J, lam


# ---------------------------------------------------------------- MATLAB Burgers prototypes
def _xyz(a: np.ndarray):
    """(nx, ny, nz) of an x-fastest field stored [z][y][x], [y][x] or [x]."""
    s = a.shape[::-1]
    return s[0], (s[1] if len(s) > 1 else 1), (s[2] if len(s) > 2 else 1)


def proto_residual(order: int, axis: int, u: np.ndarray, h: float, line_max: bool = False) -> np.ndarray:
    """d f(u)/d axis by WENO{order}resAdv_{X,Y,Z}.m (line_max: WENO{order}resAdv1d.m)."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    res = np.empty_like(u)
    nx, ny, nz = _xyz(u)
    lib().orc_proto_residual_f64(order, axis, int(line_max), nx, ny, nz, h, _p(u), _p(res))
    return res


def proto_run(order: int, u0: np.ndarray, h, cfl: float, tEnd: float, max_steps: int = 1 << 30):
    """The LFWENO{order}FDM{ndim}d.m solver loop from u0; returns (u, t, steps)."""
    u = np.array(u0, dtype=np.float64, copy=True, order="C")
    nx, ny, nz = _xyz(u)
    hh = (C.c_double * 3)(*(list(h) + [1.0] * (3 - len(h))))
    t = C.c_double(0.0)
    it = lib().orc_proto_run_f64(order, u.ndim, nx, ny, nz, hh, cfl, tEnd, max_steps, _p(u), C.byref(t))
    return u, t.value, int(it)


def weno7_side(f) -> float:
    a = (C.c_double * 7)(*[float(x) for x in f])
    return lib().orc_weno7_side_f64(a)


def lsrk54_gain(z: complex) -> complex:
    gr, gi = C.c_double(), C.c_double()
    lib().orc_lsrk54_gain(z.real, z.imag, C.byref(gr), C.byref(gi))
    return complex(gr.value, gi.value)
