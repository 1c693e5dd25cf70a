"""Builds the native libraries in-tree with nvcc for sm_103a (no cmake, no torch extension).

Outputs (all git-ignored) go to ``multigpu_advectiondiffusion_gb300/_lib``:

* ``libadvdiff.so``                -- the native C ABI of include/advdiff.h (+ advdiff_ref_ops.h)
* ``libadvdiff_checked.so``        -- the same with ADV_BOUNDS_CHECK (memory indices tested; for tests)
* ``libadvdiff_compat_heat2d.so``  -- the reference's 2D heat extern "C" names
* ``libadvdiff_compat_heat3d.so``  -- the reference's 3D heat extern "C" names
* ``libadvdiff_compat_burgers3d.so`` -- the reference's Burgers extern "C" names
* ``heat2d``, ``heat3d``, ``burgers3d``, ``burgers2d`` -- drivers with the reference's command lines

Translation units compile in parallel; a unit is rebuilt only when it or a header changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
OBJ = OUT / "obj"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE), "-I", str(CSRC)]

LIB_UNITS = ["api.cu", "api_device.cu", "heat_kernels.cu", "heat_f32.cu", "heat_f64.cu", "heat2_f32.cu", "burgers_f32.cu", "burgers_f64.cu",
             "ref_ops.cu", "noalloc.cu", "heat_batch.cu", "burgers_batch_f32.cu", "burgers_batch_f64.cu", "ensemble.cu",
             "heatk.cu", "burgers_adjoint.cu", "autotune.cu", "weno7.cu", "heat2d_multi.cu",
             "formats.cpp"]
# library -> (source, extra defines)
COMPAT = {
    "libadvdiff_compat_heat2d.so": ("compat_heat2d.cpp", []),
    "libadvdiff_compat_heat3d.so": ("compat_heat3d.cpp", []),
    "libadvdiff_compat_burgers3d.so": ("compat_burgers3d.cpp", []),
    "libadvdiff_compat_heat2d_pitched.so": ("compat_heat2d.cpp", ["-DADV_COMPAT_PITCHED"]),
    "libadvdiff_compat_heat3d_pitched.so": ("compat_heat3d.cpp", ["-DADV_COMPAT_PITCHED"]),
    "libadvdiff_compat_burgers3d_pitched.so": ("compat_burgers3d.cpp", ["-DADV_COMPAT_PITCHED"]),
    "libadvdiff_compat_heat3d_blocking.so": ("compat_heat3d.cpp", ["-DADV_COMPAT_BLOCKING"]),
    "libadvdiff_compat_burgers3d_sharedmem.so": ("compat_burgers3d.cpp",
                                                 ["-DADV_COMPAT_PITCHED", "-DADV_COMPAT_SHAREDMEM"]),
}
DRIVERS = {"heat2d": "drivers/heat2d_main.cpp", "heat3d": "drivers/heat3d_main.cpp",
           "burgers3d": "drivers/burgers3d_main.cpp", "burgers2d": "drivers/burgers2d_main.cpp"}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build the library")
    return exe


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _stale(target: Path, sources: list[Path], hdr: float) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources) or hdr > t


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    OBJ.mkdir(parents=True, exist_ok=True)
    nv = nvcc()
    hdr = _headers_mtime()
    jobs = jobs or max(2, min(8, os.cpu_count() or 2))

    def compile_unit(src: Path, defines: list[str] = (), tag: str = "") -> Path:
        obj = OBJ / (src.name + tag + ".o")
        if _stale(obj, [src], hdr):
            lang = ["-x", "cu"] if src.suffix == ".cu" else []
            cmd = [nv, *ARCH, *NVCC_FLAGS, *defines, *lang, "-c", str(src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), flush=True)
            _run(cmd)
        return obj

    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(compile_unit, [CSRC / u for u in LIB_UNITS]))
        checked_objs = list(ex.map(lambda u: compile_unit(CSRC / u, ["-DADV_BOUNDS_CHECK"], ".checked"), LIB_UNITS))
        compat_objs = dict(zip(COMPAT, ex.map(lambda kv: compile_unit(CSRC / kv[1][0], kv[1][1], "." + kv[0]),
                                              COMPAT.items())))
        driver_objs = dict(zip(DRIVERS, ex.map(compile_unit, [CSRC / s for s in DRIVERS.values()])))

    lib = OUT / "libadvdiff.so"
    if _stale(lib, objs, 0.0):
        _run([nv, *ARCH, "-shared", "-cudart", "shared", "-o", str(lib), *map(str, objs)])
    # the bounds-checked build (ADV_BOUNDS_CHECK: every global index of the stage kernels and the
    # reference operators tested before use), for the tests; internal references bind to itself
    checked = OUT / "libadvdiff_checked.so"
    if _stale(checked, checked_objs, 0.0):
        _run([nv, *ARCH, "-shared", "-cudart", "shared", "-Xlinker", "-Bsymbolic", "-o", str(checked),
              *map(str, checked_objs)])
    rpath = ["-Xlinker", "-rpath,$ORIGIN"]
    for name, obj in compat_objs.items():
        target = OUT / name
        if _stale(target, [obj, lib], 0.0):
            _run([nv, *ARCH, "-shared", "-cudart", "shared", "-o", str(target), str(obj), "-L", str(OUT), "-ladvdiff", *rpath])
    for name, obj in driver_objs.items():
        target = OUT / name
        if _stale(target, [obj, lib], 0.0):
            _run([nv, *ARCH, "-cudart", "shared", "-o", str(target), str(obj), "-L", str(OUT), "-ladvdiff", *rpath])
    return lib


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", OUT)
