"""The reference's single-GPU CUDA kernels, run on the GPU as the reference's drivers run them.

TEST INFRASTRUCTURE (part of the oracle): used only by the GPU parity tests and by the benchmark's
reference arm, never by the library. The kernels are the reference's own sources compiled by
oracle/ref_build.py into cubins (oracle/_ref/); this module loads them with the CUDA driver API
(ctypes on libcuda), sets their __constant__ coefficients and launches them with the reference's
launch geometry in the order of the reference's host loops:

  heat3d_run   SingleGPU/Diffusion3d_baselineCode/main.cpp:95-122 (D2D copy u -> uo, then per
               RK stage Compute_Laplace3d + Compute_RK); scheme "o2-euler" swaps in the
               reference's Compute_Laplace3d_O2 (kernels.cu:37-64) and runs RK stage 1 only.
  heat2d_run   SingleGPU/Diffusion2d/main.cpp:97-125.
  burgers3d_run SingleGPU/Burgers3d_WENO5/main.cpp:88-150 (dt = min(CFL dx, diffusive bound),
               trimmed to tEnd; per RK stage Compute_dF, dG, dH, Compute_Laplace_Async, Compute_RK).
  heat3d_blocking_run SingleGPU/Diffusion3d_Blocking/main.cpp:86-123 (Lu zeroed once; per RK
               stage Compute_Laplace3d_Async over 16-plane z blocks from kstart 3 to kstop nz-2,
               then Compute_RK).

Launch safety, checked by reading the kernels: Compute_Laplace2d writes Lu on every thread that
fails its interior test (SingleGPU/Diffusion2d/kernels.cu:86-87), including threads of partial
blocks past the array, so heat2d_run requires nx and ny to be multiples of the block;
Compute_Laplace_Async starts its first slab at max(3, blockIdx.z*16) without testing it against
kstop (SingleGPU/Burgers3d_WENO5/kernels.cu:458-471), which reads past the array when
nz mod 16 is 1 or 2, so burgers3d_run rejects those nz; Compute_dF/dG take x- and y-extents
from swapped grids (main.cpp:101,105), so burgers3d_run requires nx == ny == nz and equal
block sizes. The blocked heat kernel likewise starts each z block at max(3, 16*blockIdx.z)
without the kstop test (SingleGPU/Diffusion3d_Blocking/kernels.cu:57-68), reading two planes past
that plane, so heat3d_blocking_run rejects nz mod 16 of 1 or 2 (the last block's first plane is
then nz-2 or nz-1). Every state array is FP64 (the reference's REAL).
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

REF = Path(__file__).resolve().parent / "_ref"

_cu = None


def _driver():
    global _cu
    if _cu is None:
        lib = C.CDLL("libcuda.so.1")
        for name in ("cuModuleLoadData", "cuModuleUnload", "cuModuleGetFunctionCount", "cuModuleEnumerateFunctions",
                     "cuFuncGetName", "cuModuleGetGlobal_v2", "cuMemcpyHtoD_v2", "cuLaunchKernel",
                     "cuMemcpyDtoDAsync_v2", "cuMemsetD8Async"):
            getattr(lib, name).restype = C.c_int
        _check(lib.cuInit(0), "cuInit")
        _cu = lib
    return _cu


def _check(r: int, what: str) -> None:
    if r != 0:
        raise RuntimeError(f"{what}: CUresult {r}")


def available(name: str = "heat3d") -> bool:
    return (REF / f"{name}.cubin").exists()


def _plain(mangled: str) -> str:
    """Function name of an Itanium-mangled free function (_Z<len><name>...)."""
    if not mangled.startswith("_Z"):
        return mangled
    i = 2
    j = i
    while j < len(mangled) and mangled[j].isdigit():
        j += 1
    n = int(mangled[i:j])
    return mangled[j:j + n]


class RefModule:
    """One reference cubin loaded into the current (torch primary) context."""

    def __init__(self, name: str, nofma: bool = False):
        import torch
        torch.zeros(1, device="cuda")  # make the primary context current in this thread
        path = REF / f"{name}{'_nofma' if nofma else ''}.cubin"
        if not path.exists():
            raise FileNotFoundError(f"{path} is missing: run oracle/ref_build.py where the reference sources are")
        cu = _driver()
        self._img = C.create_string_buffer(path.read_bytes())
        self.mod = C.c_void_p()
        _check(cu.cuModuleLoadData(C.byref(self.mod), self._img), f"load {path.name}")
        n = C.c_uint(0)
        _check(cu.cuModuleGetFunctionCount(C.byref(n), self.mod), "function count")
        fns = (C.c_void_p * n.value)()
        _check(cu.cuModuleEnumerateFunctions(fns, n, self.mod), "enumerate functions")
        self.fn = {}
        for f in fns:
            nm = C.c_char_p()
            _check(cu.cuFuncGetName(C.byref(nm), C.c_void_p(f)), "function name")
            self.fn[_plain(nm.value.decode())] = C.c_void_p(f)

    def set_const(self, name: str, value: float) -> None:
        cu = _driver()
        dptr, size = C.c_uint64(0), C.c_size_t(0)
        _check(cu.cuModuleGetGlobal_v2(C.byref(dptr), C.byref(size), self.mod, name.encode()), f"symbol {name}")
        v = C.c_double(value)
        _check(cu.cuMemcpyHtoD_v2(dptr, C.byref(v), C.c_size_t(8)), f"set {name}")

    def launch(self, name: str, grid, block, args, stream: int) -> None:
        ptrs = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        _check(_driver().cuLaunchKernel(self.fn[name], C.c_uint(grid[0]), C.c_uint(grid[1]), C.c_uint(grid[2]),
                                        C.c_uint(block[0]), C.c_uint(block[1]), C.c_uint(block[2]), C.c_uint(0),
                                        C.c_void_p(stream), ptrs, None), f"launch {name}")

    def close(self) -> None:
        if self.mod:
            _driver().cuModuleUnload(self.mod)
            self.mod = None


def _div(a: int, b: int) -> int:
    return (a + b - 1) // b


def _copy(dst, src, stream: int) -> None:
    _check(_driver().cuMemcpyDtoDAsync_v2(C.c_uint64(dst.data_ptr()), C.c_uint64(src.data_ptr()),
                                          C.c_size_t(src.numel() * src.element_size()), C.c_void_p(stream)), "D2D")


def _stream() -> int:
    import torch
    return torch.cuda.current_stream().cuda_stream


def heat3d_run(mod: RefModule, u, nx: int, ny: int, nz: int, kx: float, ky: float, kz: float, dt: float,
               iters: int, block=(32, 4, 4), scheme: str = "o4-rk3") -> None:
    """iters time steps in place on the FP64 CUDA tensor u. kx, ky, kz are the reference's
    __constant__ coefficients C/(12 h^2) (the O2 kernel multiplies them by 12)."""
    import torch
    assert u.dtype == torch.float64 and u.numel() == nx * ny * nz
    s = _stream()
    uo = torch.empty_like(u)
    Lu = torch.zeros_like(u)
    for n, v in (("d_kx", kx), ("d_ky", ky), ("d_kz", kz)):
        mod.set_const(n, v)
    grid = (_div(nx, block[0]), _div(ny, block[1]), _div(nz, block[2]))
    lap = "Compute_Laplace3d_O2" if scheme == "o2-euler" else "Compute_Laplace3d"
    stages = (1,) if scheme == "o2-euler" else (1, 2, 3)
    up, uop, lp = C.c_void_p(u.data_ptr()), C.c_void_p(uo.data_ptr()), C.c_void_p(Lu.data_ptr())
    dims = [C.c_uint(nx), C.c_uint(ny), C.c_uint(nz)]
    for _ in range(iters):
        _copy(uo, u, s)
        for st in stages:
            mod.launch(lap, grid, block, [up, lp, *dims], s)
            mod.launch("Compute_RK", grid, block, [up, uop, lp, C.c_uint(st), *dims, C.c_double(dt)], s)


def heat3d_blocking_run(mod: RefModule, u, nx: int, ny: int, nz: int, kx: float, ky: float, kz: float, dt: float,
                        iters: int) -> None:
    """iters time steps in place on the dense FP64 CUDA tensor u (pitch = nx), with the blocked
    program's launch geometry: Laplacian blocks (32, 4, 1) over (nx/32, ny/4, nz/16), RK blocks
    (32, 4, 4) over (nx/32, ny/4, nz/4) (main.cpp:88-98)."""
    import torch
    assert u.dtype == torch.float64 and u.numel() == nx * ny * nz
    if nz % 16 in (1, 2) or min(nx, ny, nz) < 7:
        raise ValueError("the blocked Laplacian's last z block would read past the array")
    s = _stream()
    uo = torch.empty_like(u)
    Lu = torch.zeros_like(u)
    for n, v in (("d_kx", kx), ("d_ky", ky), ("d_kz", kz)):
        mod.set_const(n, v)
    g2, b2 = (_div(nx, 32), _div(ny, 4), _div(nz, 16)), (32, 4, 1)
    g3, b3 = (_div(nx, 32), _div(ny, 4), _div(nz, 4)), (32, 4, 4)
    up, uop, lp = C.c_void_p(u.data_ptr()), C.c_void_p(uo.data_ptr()), C.c_void_p(Lu.data_ptr())
    dims = [C.c_uint(nx), C.c_uint(nx), C.c_uint(ny), C.c_uint(nz)]  # pitch, nx, ny, nz
    for _ in range(iters):
        _copy(uo, u, s)
        for st in (1, 2, 3):
            mod.launch("Compute_Laplace3d_Async", g2, b2, [up, lp, *dims, C.c_uint(3), C.c_uint(nz - 2), C.c_uint(16)],
                       s)
            mod.launch("Compute_RK", g3, b3, [up, uop, lp, C.c_uint(st), *dims, C.c_double(dt)], s)


def heat2d_run(mod: RefModule, u, nx: int, ny: int, kx: float, ky: float, dt: float, iters: int,
               block=(32, 8)) -> None:
    import torch
    assert u.dtype == torch.float64 and u.numel() == nx * ny
    if nx % block[0] or ny % block[1]:
        raise ValueError("the reference's Compute_Laplace2d writes past the array on partial blocks: "
                         "nx and ny must be multiples of the block")
    s = _stream()
    uo = torch.empty_like(u)
    Lu = torch.zeros_like(u)
    mod.set_const("d_kx", kx)
    mod.set_const("d_ky", ky)
    grid = (nx // block[0], ny // block[1], 1)
    b3 = (block[0], block[1], 1)
    up, uop, lp = C.c_void_p(u.data_ptr()), C.c_void_p(uo.data_ptr()), C.c_void_p(Lu.data_ptr())
    for _ in range(iters):
        _copy(uo, u, s)
        for st in (1, 2, 3):
            mod.launch("Compute_Laplace2d", grid, b3, [up, lp, C.c_uint(nx), C.c_uint(ny)], s)
            mod.launch("Compute_RK", grid, b3, [up, uop, lp, C.c_uint(st), C.c_uint(nx), C.c_uint(ny),
                                                  C.c_double(dt)], s)


def burgers3d_run(mod: RefModule, u, n: int, L: float, tEnd: float, cfl: float, C_visc: float = 1e-5,
                  block: int = 8, max_steps: int | None = None) -> tuple[float, int]:
    """The reference's Burgers loop on an n^3 node grid of [0,L]^3 (dx = L/(n-1)); returns (t, steps)."""
    import torch
    assert u.dtype == torch.float64 and u.numel() == n ** 3
    if n % 16 in (1, 2):
        raise ValueError("the reference's Compute_Laplace_Async reads past the array when nz mod 16 is 1 or 2")
    s = _stream()
    dx = L / (n - 1)
    k = C_visc / (12 * dx * dx)
    for name in ("d_kx", "d_ky", "d_kz"):
        mod.set_const(name, k)
    uo = torch.empty_like(u)
    Lu = torch.zeros_like(u)
    b = block
    g = _div(n, b)
    grid3, blk3 = (g, g, g), (b, b, b)
    grid2, blk2 = (g, g, 1), (b, b, 1)
    gridA, blkA = (_div(n, 64), _div(n, 4), _div(n, 16)), (64, 4, 1)
    up, uop, lp = C.c_void_p(u.data_ptr()), C.c_void_p(uo.data_ptr()), C.c_void_p(Lu.data_ptr())
    dims = [C.c_uint(n), C.c_uint(n), C.c_uint(n)]
    h = C.c_double(dx)
    t, it = 0.0, 0
    dy = dz = dx
    dt2 = 1.0 / (2 * C_visc * (1 / dx / dx + 1 / dy / dy + 1 / dz / dz)) * 0.9 if C_visc > 0 else math.inf
    while t < tEnd and (max_steps is None or it < max_steps):
        dt1 = cfl * dx / 1.0
        dt = dt1 if dt1 < dt2 else dt2
        if t + dt > tEnd:
            dt = tEnd - t
        t += dt
        it += 1
        _copy(uo, u, s)
        for st in (1, 2, 3):
            mod.launch("Compute_dF", grid2, blk2, [up, lp, *dims, h], s)
            mod.launch("Compute_dG", grid2, blk2, [up, lp, *dims, h], s)
            mod.launch("Compute_dH", grid2, blk2, [up, lp, *dims, h], s)
            mod.launch("Compute_Laplace_Async", gridA, blkA,
                       [up, lp, C.c_uint(n), *dims, C.c_uint(3), C.c_uint(n - 2), C.c_uint(16)], s)
            mod.launch("Compute_RK", grid3, blk3, [up, uop, lp, C.c_uint(st), *dims, C.c_double(dt)], s)
    return t, it
