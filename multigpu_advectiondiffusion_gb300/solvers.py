"""Host-side mirror of the reference's solver surface over the CUDA library.

The reference drives its kernels from main.cpp time loops (SingleGPU/Diffusion3d_baselineCode/
main.cpp:55-122, SingleGPU/Diffusion2d/main.cpp:52-125, SingleGPU/Burgers3d_WENO5/
main.cpp:53-150). This module keeps those constants and dt rules and calls the fused stage
kernels through the C ABI on torch CUDA tensors (torch supplies device memory and streams only).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from dataclasses import dataclass

from . import _native as N


def _ptr(t) -> int:
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return t.data_ptr()


def _dtype_code(t) -> int:
    import torch
    if t.dtype == torch.float32:
        return N.ADV_F32
    if t.dtype == torch.float64:
        return N.ADV_F64
    raise ValueError(f"unsupported dtype {t.dtype}")


def _fields(numel: int, *ts) -> int:
    """Checks the grid-shaped tensors of one call and returns their dtype code. The C ABI takes
    plain pointers and cannot see sizes, so each must be a contiguous CUDA tensor of one dtype,
    on one device, with at least `numel` elements; otherwise the kernels would read or write
    past it (an FP64 state in an FP32 buffer of the same length included)."""
    first = ts[0]
    code = _dtype_code(first)
    for t in ts:
        _ptr(t)
        if t.dtype != first.dtype:
            raise ValueError(f"fields of one call must share a dtype: {first.dtype} and {t.dtype}")
        if t.device != first.device:
            raise ValueError(f"fields of one call must share a device: {first.device} and {t.device}")
        if t.numel() < numel:
            raise ValueError(f"a field has {t.numel()} elements; the grid has {numel}")
    return code


def _stream(stream, like):
    """Stream handle of a call: the caller's stream if given, else torch's current stream on the
    device of `like` (so the library's work is ordered with the caller's torch work, also under
    `with torch.cuda.stream(...)`); None (the default stream) without CUDA."""
    if stream is not None:
        return N.stream_handle(stream)
    import torch
    if getattr(like, "is_cuda", False) and torch.cuda.is_available():
        return torch.cuda.current_stream(like.device).cuda_stream or None
    return None


def _buffer(t, nbytes: int, what: str) -> int:
    """Pointer of a caller-supplied work buffer after checking it holds `nbytes`."""
    p = _ptr(t)
    if t.numel() * t.element_size() < nbytes:
        raise ValueError(f"{what} has {t.numel() * t.element_size()} bytes; {nbytes} are needed")
    return p


@dataclass
class HeatConfig:
    """Heat-equation scheme (fields as adv_heat_desc in include/advdiff.h)."""
    ndim: int
    nx: int
    ny: int
    nz: int
    order: int = 4
    frozen: int = 2
    zero_boundary: bool = False
    kx: float = 0.0
    ky: float = 0.0
    kz: float = 0.0
    dt: float = 0.0
    time: int = N.ADV_SSPRK3
    contract: bool = False  # FP64 only: the fused multiply-add form instead of the reference's rounding

    @classmethod
    def reference_3d(cls, C: float, L: int, W: int, H: int, nx: int, ny: int, nz: int) -> "HeatConfig":
        """The reference 3D scheme: O4 + SSP-RK3, dt = 0.9/(2C sum 1/h^2), k = C/(12 h^2), two
        frozen layers (SingleGPU/Diffusion3d_baselineCode/main.cpp:55-62, kernels.cu:127)."""
        dx, dy, dz = L / (nx - 1), W / (ny - 1), H / (nz - 1)
        dt = 1 / (2 * C * (1 / dx / dx + 1 / dy / dy + 1 / dz / dz)) * 0.9
        return cls(3, nx, ny, nz, 4, 2, False, C / (12 * dx * dx), C / (12 * dy * dy), C / (12 * dz * dz), dt)

    @classmethod
    def reference_2d(cls, C: float, L: int, W: int, nx: int, ny: int) -> "HeatConfig":
        """The reference 2D scheme: O4 + SSP-RK3, three frozen layers
        (SingleGPU/Diffusion2d/main.cpp:52-57, kernels.cu:53)."""
        dx, dy = L / (nx - 1), W / (ny - 1)
        dt = 1 / (2 * C * (1 / dx / dx + 1 / dy / dy)) * 0.9
        return cls(2, nx, ny, 1, 4, 3, False, C / (12 * dx * dx), C / (12 * dy * dy), 0.0, dt)

    @classmethod
    def dirichlet_o2(cls, ndim: int, n: int, k: float = 1.0, r: float | None = None, L: float = 1.0) -> "HeatConfig":
        """O2 (5/7-point) forward Euler with r = k dt/h^2 on the node grid of [0,L]^d, u = 0 on the
        boundary nodes. Default r: 0.2 in 2D, 1/8 in 3D."""
        r = (0.2 if ndim == 2 else 0.125) if r is None else r
        h = L / (n - 1)
        c = k / (h * h)
        return cls(ndim, n, n, n if ndim == 3 else 1, 2, 1, True, c, c, c if ndim == 3 else 0.0, r * h * h / k,
                   N.ADV_EULER)

    def desc(self, dtype: int) -> N.HeatDesc:
        return N.HeatDesc(self.ndim, self.nx, self.ny, self.nz if self.ndim == 3 else 1, dtype, self.order,
                          self.frozen, int(self.zero_boundary), self.kx, self.ky, self.kz, self.dt,
                          int(self.contract), 0)

    @property
    def numel(self) -> int:
        return self.nx * self.ny * (self.nz if self.ndim == 3 else 1)


def heat_stage(cfg: HeatConfig, stage: int, u_in, u_n, u_out, stream=None) -> None:
    """One fused stage u_out = combine(u_n, u_in + dt L(u_in)) (adv_heat_stage)."""
    d = cfg.desc(_fields(cfg.numel, u_in, u_n, u_out))
    N.check(N.load().adv_heat_stage(C.byref(d), stage, _ptr(u_in), _ptr(u_n), _ptr(u_out), _stream(stream, u_in)),
            "adv_heat_stage")


def _heat_workspace_bytes(cfg: HeatConfig, dtype: int) -> int:
    d = cfg.desc(dtype)
    nb = C.c_size_t(0)
    N.check(N.load().adv_heat_workspace_bytes(C.byref(d), cfg.time, C.byref(nb)), "adv_heat_workspace_bytes")
    return nb.value


def heat_workspace(cfg: HeatConfig, like):
    import torch
    return torch.empty(_heat_workspace_bytes(cfg, _dtype_code(like)), dtype=torch.uint8, device=like.device)


def heat_run(cfg: HeatConfig, u, nsteps: int, workspace=None, stream=None):
    """nsteps time steps in place on u (adv_heat_run); returns u."""
    code = _fields(cfg.numel, u)
    ws = heat_workspace(cfg, u) if workspace is None else workspace
    wp = _buffer(ws, _heat_workspace_bytes(cfg, code), "the heat workspace")
    d = cfg.desc(code)
    N.check(N.load().adv_heat_run(C.byref(d), cfg.time, int(nsteps), _ptr(u), wp, _stream(stream, u)),
            "adv_heat_run")
    return u


@dataclass
class BurgersConfig:
    """Burgers scheme (fields as adv_burgers_desc in include/advdiff.h)."""
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    weno: int = N.ADV_WENO5_Z
    lf: int = N.ADV_LF_LOCAL
    bc: int = N.ADV_BC_FROZEN
    div: int = N.ADV_DIV_F32
    bug_b2: bool = False
    C: float = 0.0

    @classmethod
    def reference(cls, L: float, W: float, H: float, nx: int, ny: int, nz: int, C: float = 1e-5,
                  bug_b2: bool = False) -> "BurgersConfig":
        """The reference scheme: node grid dx = L/(N-1), local LF, WENO5-Z, viscous term C = 1e-5,
        frozen 3 layers (SingleGPU/Burgers3d_WENO5/main.cpp:53-59)."""
        return cls(nx, ny, nz, L / (nx - 1), W / (ny - 1), H / (nz - 1), N.ADV_WENO5_Z, N.ADV_LF_LOCAL,
                   N.ADV_BC_FROZEN, N.ADV_DIV_F32, bug_b2, C)

    @classmethod
    def periodic(cls, n: int, L: float = 2.0, weno: str = "z", lf: str = "global",
                 div: str | int = "f32") -> "BurgersConfig":
        """Inviscid periodic [0,L)^3 on n^3 cell centres, dx = L/n. div: "f32", "f64", "fast" or an
        adv_div code."""
        h = L / n
        if isinstance(div, str):
            div = {"f32": N.ADV_DIV_F32, "f64": N.ADV_DIV_F64, "fast": N.ADV_DIV_FAST}[div]
        return cls(n, n, n, h, h, h, N.ADV_WENO5_Z if weno == "z" else N.ADV_WENO5_JS,
                   N.ADV_LF_GLOBAL if lf == "global" else N.ADV_LF_LOCAL, N.ADV_BC_PERIODIC, int(div), False, 0.0)

    @classmethod
    def reference_2d(cls, L: float, W: float, nx: int, ny: int, C: float = 0.0) -> "BurgersConfig":
        """The reference's 2D Burgers scheme on one plane (nz = 1): node grid dx = L/(N-1), local
        LF, WENO5-JS, inviscid (MultiGPU/Burgers2d_Baseline/main.c:58, Kernels.cu:112-222), with
        three frozen layers in x and y."""
        return cls(nx, ny, 1, L / (nx - 1), W / (ny - 1), L / (nx - 1), N.ADV_WENO5_JS, N.ADV_LF_LOCAL,
                   N.ADV_BC_FROZEN, N.ADV_DIV_F32, False, C)

    def desc(self, dtype: int) -> N.BurgersDesc:
        k = [self.C / (12 * h * h) if self.C else 0.0 for h in (self.dx, self.dy, self.dz)]
        if self.nz == 1:  # 2D: no z term
            k[2] = 0.0
        return N.BurgersDesc(self.nx, self.ny, self.nz, dtype, self.weno, self.lf, self.bc, self.div,
                             int(self.bug_b2), 0, self.dx, self.dy, self.dz, *k)

    @property
    def numel(self) -> int:
        return self.nx * self.ny * self.nz


def burgers_stage(cfg: BurgersConfig, stage: int, u_in, u_n, u_out, dt: float, alpha: float = 0.0,
                  maxabs_key=None, stream=None) -> None:
    """One fused SSP-RK3 stage (adv_burgers_stage). maxabs_key: optional device tensor of one
    int32 (FP32 state) / int64 (FP64 state), zeroed by the caller, receiving max|u_out| bits."""
    code = _fields(cfg.numel, u_in, u_n, u_out)
    d = cfg.desc(code)
    key = None
    if maxabs_key is not None:
        key = _buffer(maxabs_key, u_in.element_size(), "maxabs_key")
        if maxabs_key.element_size() != u_in.element_size():
            raise ValueError("maxabs_key must be int32 for an FP32 state and int64 for an FP64 state")
    N.check(N.load().adv_burgers_stage(C.byref(d), stage, _ptr(u_in), _ptr(u_n), _ptr(u_out), float(dt), float(alpha),
                                       key, _stream(stream, u_in)), "adv_burgers_stage")


def _burgers_workspace_bytes(cfg: BurgersConfig, dtype: int) -> int:
    d = cfg.desc(dtype)
    nb = C.c_size_t(0)
    N.check(N.load().adv_burgers_workspace_bytes(C.byref(d), C.byref(nb)), "adv_burgers_workspace_bytes")
    return nb.value


def burgers_workspace(cfg: BurgersConfig, like):
    import torch
    return torch.empty(_burgers_workspace_bytes(cfg, _dtype_code(like)), dtype=torch.uint8, device=like.device)


def burgers_run(cfg: BurgersConfig, u, tEnd: float, cfl: float, dt_rule: int = N.ADV_DT_MAXU,
                max_steps: int = 1 << 40, workspace=None, stream=None) -> tuple[float, int]:
    """Time loop to tEnd in place on u (adv_burgers_run); returns (t, steps)."""
    code = _fields(cfg.numel, u)
    ws = burgers_workspace(cfg, u) if workspace is None else workspace
    wp = _buffer(ws, _burgers_workspace_bytes(cfg, code), "the Burgers workspace")
    d = cfg.desc(code)
    t = C.c_double(0.0)
    steps = C.c_int64(0)
    N.check(N.load().adv_burgers_run(C.byref(d), _ptr(u), wp, float(tEnd), float(cfl), int(dt_rule),
                                     float(cfg.C), int(max_steps), C.byref(t), C.byref(steps),
                                     _stream(stream, u)), "adv_burgers_run")
    return t.value, steps.value


def max_abs(u, stream=None) -> float:
    out = C.c_double(0.0)
    N.check(N.load().adv_max_abs(_dtype_code(u), _ptr(u), u.numel(), C.byref(out), _stream(stream, u)),
            "adv_max_abs")
    return out.value


@dataclass
class Weno7Config:
    """The seventh-order WENO prototype solver (adv_weno7_desc): a 2D (nz = 1) or 3D node grid with
    spacings dx, dy, dz."""
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float

    def desc(self, dtype: int) -> N.Weno7Desc:
        return N.Weno7Desc(self.nx, self.ny, self.nz, dtype, self.dx, self.dy, self.dz)

    @property
    def numel(self) -> int:
        return self.nx * self.ny * self.nz


def _weno7_workspace_bytes(cfg: Weno7Config, code: int) -> int:
    nb = C.c_size_t(0)
    N.check(N.load().adv_weno7_workspace_bytes(C.byref(cfg.desc(code)), C.byref(nb)), "adv_weno7_workspace_bytes")
    return nb.value


def weno7_workspace(cfg: Weno7Config, like):
    import torch
    return torch.empty(_weno7_workspace_bytes(cfg, _dtype_code(like)), dtype=torch.uint8, device=like.device)


def weno7_rhs(cfg: Weno7Config, u, L, workspace=None, stream=None) -> None:
    """L = the summed prototype residuals of u (adv_weno7_rhs)."""
    code = _fields(cfg.numel, u, L)
    ws = weno7_workspace(cfg, u) if workspace is None else workspace
    wp = _buffer(ws, _weno7_workspace_bytes(cfg, code), "the WENO7 workspace")
    N.check(N.load().adv_weno7_rhs(C.byref(cfg.desc(code)), _ptr(u), _ptr(L), wp, _stream(stream, u)), "adv_weno7_rhs")


def weno7_run(cfg: Weno7Config, u, tEnd: float, cfl: float, max_steps: int = 1 << 40, workspace=None,
              stream=None) -> tuple[float, int]:
    """The prototype's LSRK(5,4) time loop to tEnd in place on u (adv_weno7_run); returns (t, steps)."""
    code = _fields(cfg.numel, u)
    ws = weno7_workspace(cfg, u) if workspace is None else workspace
    wp = _buffer(ws, _weno7_workspace_bytes(cfg, code), "the WENO7 workspace")
    t = C.c_double(0.0)
    steps = C.c_int64(0)
    N.check(N.load().adv_weno7_run(C.byref(cfg.desc(code)), _ptr(u), wp, float(tEnd), float(cfl), int(max_steps),
                                   C.byref(t), C.byref(steps), _stream(stream, u)), "adv_weno7_run")
    return t.value, steps.value


@dataclass
class HeatKConfig:
    """3D heat with a diffusivity field (adv_heatk_desc): c_a = dt / h_a^2."""
    nx: int
    ny: int
    nz: int
    cx: float
    cy: float
    cz: float
    zero_boundary: bool = True

    @classmethod
    def cube(cls, n: int, dt_kmax_over_h2: float, k_max: float, L: float = 1.0) -> "HeatKConfig":
        """n^3 nodes on [0,L]^3, dt chosen so dt k_max / h^2 = dt_kmax_over_h2 (<= 1/6 is stable)."""
        c = dt_kmax_over_h2 / k_max
        return cls(n, n, n, c, c, c, True)

    def desc(self, dtype: int) -> N.HeatKDesc:
        return N.HeatKDesc(self.nx, self.ny, self.nz, dtype, int(self.zero_boundary), 0, self.cx, self.cy, self.cz)

    @property
    def numel(self) -> int:
        return self.nx * self.ny * self.nz


def heatk_step(cfg: HeatKConfig, k, u_in, u_out, stream=None) -> None:
    d = cfg.desc(_fields(cfg.numel, u_in, k, u_out))
    N.check(N.load().adv_heatk_step(C.byref(d), _ptr(k), _ptr(u_in), _ptr(u_out), _stream(stream, u_in)),
            "adv_heatk_step")


def heatk_adjoint_step(cfg: HeatKConfig, k, u_n, lam_next, lam_out, grad_k, stream=None) -> None:
    d = cfg.desc(_fields(cfg.numel, u_n, k, lam_next, lam_out, grad_k))
    N.check(N.load().adv_heatk_adjoint_step(C.byref(d), _ptr(k), _ptr(u_n), _ptr(lam_next), _ptr(lam_out),
                                            _ptr(grad_k), _stream(stream, u_n)), "adv_heatk_adjoint_step")


def _heatk_buffers(cfg, like, nsteps, interval):
    import torch
    d = cfg.desc(_dtype_code(like))
    cb, wb = C.c_size_t(0), C.c_size_t(0)
    N.check(N.load().adv_heatk_checkpoint_bytes(C.byref(d), int(nsteps), int(interval), C.byref(cb), C.byref(wb)),
            "adv_heatk_checkpoint_bytes")
    return (torch.empty(cb.value, dtype=torch.uint8, device=like.device),
            torch.empty(wb.value, dtype=torch.uint8, device=like.device))


def default_interval(nsteps: int) -> int:
    """sqrt(N) checkpoint spacing: about sqrt(N) checkpoints plus sqrt(N) recomputed states."""
    return max(1, math.ceil(math.sqrt(max(nsteps, 1))))


def checkpoint_interval(nsteps: int, arrays_per_step: int, array_bytes: int, free_bytes: int) -> int:
    """Checkpoint spacing of a differentiable run. The whole run is kept (interval = nsteps: the
    forward run leaves every state or stage input in its work buffer and the backward run
    recomputes nothing) when its arrays_per_step * nsteps arrays fit in half of free_bytes (the
    device's free memory); otherwise sqrt(N) spacing."""
    nsteps = max(int(nsteps), 1)
    if arrays_per_step * nsteps * array_bytes <= free_bytes // 2:
        return nsteps
    return default_interval(nsteps)


def auto_interval(nsteps: int, arrays_per_step: int, like, need_grad: bool = True) -> int:
    """checkpoint_interval for a run on like's device; sqrt(N) when no gradient will be taken
    (the kept run would only cost memory)."""
    if not need_grad:
        return default_interval(nsteps)
    import torch
    free, _ = torch.cuda.mem_get_info(like.device)
    one = (like.numel() * like.element_size() + 255) // 256 * 256
    return checkpoint_interval(nsteps, arrays_per_step, one, free)


def _autograd():
    import torch

    class HeatKRun(torch.autograd.Function):
        """u(T) = heat-with-k(x) forward run from (k, u0); backward by the hand-written adjoint
        (adv_heatk_backward) over checkpoints every `interval` steps."""

        @staticmethod
        def forward(ctx, k, u0, cfg, nsteps, interval):
            u = u0.detach().clone()
            d = cfg.desc(_fields(cfg.numel, u, k))
            ckpt, work = _heatk_buffers(cfg, u, nsteps, interval)
            N.check(N.load().adv_heatk_forward(C.byref(d), _ptr(k), _ptr(u), int(nsteps), int(interval), _ptr(ckpt),
                                               _ptr(work), N.stream_handle(torch.cuda.current_stream())),
                    "adv_heatk_forward")
            ctx.save_for_backward(k)
            ctx.cfg, ctx.nsteps, ctx.interval, ctx.ckpt, ctx.work = cfg, nsteps, interval, ckpt, work
            return u

        @staticmethod
        def backward(ctx, grad_u):
            (k,) = ctx.saved_tensors
            lam = grad_u.detach().clone().contiguous()
            gk = torch.zeros_like(k)
            d = ctx.cfg.desc(_fields(ctx.cfg.numel, lam, k, gk))
            # the forward run left its last interval's states in ctx.work, untouched since
            N.check(N.load().adv_heatk_backward(C.byref(d), _ptr(k), int(ctx.nsteps), int(ctx.interval),
                                                _ptr(ctx.ckpt), _ptr(lam), _ptr(gk), _ptr(ctx.work),
                                                N.ADV_HEATK_LAST_INTERVAL_IN_WORK,
                                                N.stream_handle(torch.cuda.current_stream())), "adv_heatk_backward")
            return gk, lam, None, None, None

    return HeatKRun


def _burgers_autograd():
    import torch

    class BurgersRun(torch.autograd.Function):
        """u(T) of nsteps fixed-dt SSP-RK3 steps (periodic, local LF) from u0; backward by the
        hand-written adjoint (adv_burgers_backward) over checkpoints every `interval` steps."""

        @staticmethod
        def forward(ctx, u0, cfg, dt, nsteps, interval):
            u = u0.detach().clone()
            d = cfg.desc(_fields(cfg.numel, u))
            cb, wb = C.c_size_t(0), C.c_size_t(0)
            N.check(N.load().adv_burgers_checkpoint_bytes(C.byref(d), int(nsteps), int(interval), C.byref(cb),
                                                          C.byref(wb)), "adv_burgers_checkpoint_bytes")
            ckpt = torch.empty(cb.value, dtype=torch.uint8, device=u.device)
            work = torch.empty(wb.value, dtype=torch.uint8, device=u.device)
            N.check(N.load().adv_burgers_forward(C.byref(d), _ptr(u), float(dt), int(nsteps), int(interval),
                                                 _ptr(ckpt), _ptr(work),
                                                 N.stream_handle(torch.cuda.current_stream())), "adv_burgers_forward")
            ctx.cfg, ctx.dt, ctx.nsteps, ctx.interval, ctx.ckpt, ctx.work = cfg, dt, nsteps, interval, ckpt, work
            return u

        @staticmethod
        def backward(ctx, grad_u):
            lam = grad_u.detach().clone().contiguous()
            d = ctx.cfg.desc(_fields(ctx.cfg.numel, lam))
            # the forward run left its last interval's stage inputs in ctx.work, untouched since
            N.check(N.load().adv_burgers_backward(C.byref(d), float(ctx.dt), int(ctx.nsteps), int(ctx.interval),
                                                  _ptr(ctx.ckpt), _ptr(lam), _ptr(ctx.work),
                                                  N.ADV_BURGERS_LAST_INTERVAL_IN_WORK,
                                                  N.stream_handle(torch.cuda.current_stream())),
                    "adv_burgers_backward")
            return lam, None, None, None, None

    return BurgersRun


_BurgersRun = None


def burgers_run_fixed(cfg: BurgersConfig, u0, dt: float, nsteps: int, interval: int | None = None):
    """Differentiable (w.r.t. u0) run of nsteps fixed-dt steps; returns u(T). interval None: the
    whole run kept when its 3 stage inputs per step fit in half the free device memory (the
    backward run then recomputes nothing), else sqrt(N) checkpoints."""
    import torch
    global _BurgersRun
    if _BurgersRun is None:
        _BurgersRun = _burgers_autograd()
    if not interval:
        interval = auto_interval(nsteps, 3, u0, torch.is_grad_enabled() and u0.requires_grad)
    return _BurgersRun.apply(u0, cfg, float(dt), int(nsteps), int(interval))


def burgers_adjoint_step(cfg: BurgersConfig, u_n, u1, u2, dt: float, lam, work=None, stream=None):
    """lam (dJ/du^{n+1}) becomes dJ/du^n in place; work: 3 arrays of scratch (allocated if None)."""
    import torch
    d = cfg.desc(_fields(cfg.numel, u_n, u1, u2, lam))
    one = (cfg.numel * u_n.element_size() + 255) // 256 * 256
    if work is None:
        work = torch.empty(3 * one, dtype=torch.uint8, device=u_n.device)
    wp = _buffer(work, 3 * one, "the adjoint work buffer")
    N.check(N.load().adv_burgers_adjoint_step(C.byref(d), _ptr(u_n), _ptr(u1), _ptr(u2), float(dt), _ptr(lam),
                                              wp, _stream(stream, u_n)), "adv_burgers_adjoint_step")
    return lam


_HeatKRun = None


def heatk_run(cfg: HeatKConfig, k, u0, nsteps: int, interval: int | None = None):
    """Differentiable (w.r.t. k and u0) forward run of nsteps steps; returns u(T). interval None:
    the whole run kept when its states fit in half the free device memory (the backward run then
    recomputes nothing), else sqrt(N) checkpoints."""
    import torch
    global _HeatKRun
    if _HeatKRun is None:
        _HeatKRun = _autograd()
    if not interval:
        need = torch.is_grad_enabled() and (k.requires_grad or u0.requires_grad)
        interval = auto_interval(nsteps, 1, u0, need)
    return _HeatKRun.apply(k, u0, cfg, int(nsteps), int(interval))


class Ensemble:
    """Batched ensemble of 3D heat and Burgers problems (adv_ensemble_* in include/advdiff.h).

    heat: list of (HeatConfig, u) with u a CUDA tensor (all members: same dtype and order, 3D);
    burgers: list of (BurgersConfig, u, tEnd, cfl[, dt_rule[, max_steps]]). Each member's state
    stays in its own tensor; work buffers are allocated here. run() advances every member in
    place; burgers_result(i) gives (t, steps) of member i after the last run."""

    def __init__(self, heat=(), burgers=(), heat_time: int = N.ADV_EULER):
        import torch
        if not heat and not burgers:
            raise ValueError("an ensemble needs at least one member")
        self._lib = N.load()
        self._keep = []
        hm = (N.HeatMember * max(len(heat), 1))()
        for i, (cfg, u) in enumerate(heat):
            code = _fields(cfg.numel, u)
            ws = heat_workspace(dataclasses.replace(cfg, time=heat_time), u)
            self._keep += [u, ws]
            hm[i] = N.HeatMember(cfg.desc(code), _ptr(u), _ptr(ws))
        bm = (N.BurgersMember * max(len(burgers), 1))()
        for i, b in enumerate(burgers):
            cfg, u, tEnd, cfl = b[:4]
            dt_rule = b[4] if len(b) > 4 else N.ADV_DT_MAXU
            max_steps = b[5] if len(b) > 5 else 1 << 40
            code = _fields(cfg.numel, u)
            ws = burgers_workspace(cfg, u)
            self._keep += [u, ws]
            bm[i] = N.BurgersMember(cfg.desc(code), _ptr(u), _ptr(ws), float(tEnd), float(cfl), int(dt_rule),
                                    0, float(cfg.C), int(max_steps))
        self.n_heat, self.n_burgers = len(heat), len(burgers)
        h = C.c_void_p(None)
        with torch.cuda.device(self._keep[0].device):
            N.check(self._lib.adv_ensemble_create(hm, self.n_heat, int(heat_time), bm, self.n_burgers, C.byref(h)),
                    "adv_ensemble_create")
        self._h = h
        self.device = self._keep[0].device

    def run(self, heat_steps: int, direct: bool = False, stream=None) -> None:
        import torch
        with torch.cuda.device(self.device):
            N.check(self._lib.adv_ensemble_run(self._h, int(heat_steps), N.ADV_ENSEMBLE_DIRECT if direct else 0,
                                               _stream(stream, self._keep[0])), "adv_ensemble_run")

    def burgers_result(self, i: int) -> tuple[float, int]:
        t = C.c_double(0.0)
        steps = C.c_int64(0)
        N.check(self._lib.adv_ensemble_burgers_result(self._h, int(i), C.byref(t), C.byref(steps)),
                "adv_ensemble_burgers_result")
        return t.value, steps.value

    def shape(self) -> dict:
        hu, bu = C.c_int64(0), C.c_int64(0)
        hc, bc = C.c_int(0), C.c_int(0)
        N.check(self._lib.adv_ensemble_shape(self._h, C.byref(hu), C.byref(hc), C.byref(bu), C.byref(bc)),
                "adv_ensemble_shape")
        return {"heat_units": hu.value, "heat_ctas": hc.value, "burgers_units": bu.value, "burgers_ctas": bc.value}

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            import torch
            with torch.cuda.device(self.device):
                self._lib.adv_ensemble_destroy(self._h)
            self._h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _tune_dict(r) -> dict:
    return {"param_a": r.param_a, "param_b": r.param_b, "candidates": r.candidates, "best_us": r.best_us,
            "default_us": r.default_us}


def autotune_heat(cfg: HeatConfig, u, stream=None) -> dict:
    """Picks the heat stage's launch shape for this problem (adv_autotune_heat)."""
    r = N.TuneResult()
    d = cfg.desc(_fields(cfg.numel, u))
    N.check(N.load().adv_autotune_heat(C.byref(d), _ptr(u), _stream(stream, u), C.byref(r)), "adv_autotune_heat")
    return _tune_dict(r)


def autotune_burgers(cfg: BurgersConfig, u, stream=None) -> dict:
    """Picks the Burgers stage's launch shape for this problem (adv_autotune_burgers)."""
    r = N.TuneResult()
    d = cfg.desc(_fields(cfg.numel, u))
    N.check(N.load().adv_autotune_burgers(C.byref(d), _ptr(u), _stream(stream, u), C.byref(r)),
            "adv_autotune_burgers")
    return _tune_dict(r)


def autotune_heatk(cfg: HeatKConfig, k, u, stream=None) -> tuple[dict, dict]:
    """Picks the heat-with-k(x) step and adjoint launch shapes (adv_autotune_heatk)."""
    r1, r2 = N.TuneResult(), N.TuneResult()
    d = cfg.desc(_fields(cfg.numel, u, k))
    N.check(N.load().adv_autotune_heatk(C.byref(d), _ptr(k), _ptr(u), _stream(stream, u), C.byref(r1),
                                        C.byref(r2)), "adv_autotune_heatk")
    return _tune_dict(r1), _tune_dict(r2)


def autotune_clear() -> None:
    N.check(N.load().adv_autotune_clear(), "adv_autotune_clear")


def autotune_export() -> str:
    """The current device's tuned launch shapes as JSON text (adv_autotune_export)."""
    lib = N.load()
    n = C.c_size_t(0)
    N.check(lib.adv_autotune_export(None, 0, C.byref(n)), "adv_autotune_export")
    buf = C.create_string_buffer(n.value)
    N.check(lib.adv_autotune_export(buf, n.value, C.byref(n)), "adv_autotune_export")
    return buf.value.decode()


def autotune_import(text: str) -> None:
    """Loads shapes written by autotune_export for the current device (adv_autotune_import)."""
    N.check(N.load().adv_autotune_import(text.encode()), "adv_autotune_import")


def autotune_save(path) -> None:
    with open(path, "w") as f:
        f.write(autotune_export())


def autotune_load(path) -> None:
    with open(path) as f:
        autotune_import(f.read())


def reference_heat_final_time(dt: float, iters: int, t0: float = 0.1) -> float:
    """tFinal = t0 + dt*iters as the reference prints it (main.cpp:63)."""
    return t0 + dt * iters


def reference_burgers_fixed_dt(cfl: float, dx: float, dy: float, dz: float, C: float) -> float:
    """dt = min(CFL dx / 1, 0.9/(2C sum 1/h^2)) (SingleGPU/Burgers3d_WENO5/main.cpp:130-132)."""
    dt2 = 1.0 / (2 * C * (1 / dx / dx + 1 / dy / dy + 1 / dz / dz)) * 0.9 if C > 0 else math.inf
    return min(cfl * dx / 1.0, dt2)
