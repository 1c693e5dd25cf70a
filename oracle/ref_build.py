"""Recipe: the reference's own single-GPU CUDA kernels, compiled from its sources where they lie.

TEST INFRASTRUCTURE (part of the oracle): the outputs are device-only cubins for sm_103a under
oracle/_ref/ (git-ignored; they are GPU code, not host binaries, so they run on any host of the
GB300). oracle/ref_gpu.py loads them through the CUDA driver API and drives them with the
reference's own launch geometry and host loop. Nothing in the library loads them.

Sources (the reference checkout, read-only):
  SingleGPU/Diffusion3d_baselineCode/kernels.cu  -> heat3d       (Compute_Laplace3d[_O2], Compute_RK)
  SingleGPU/Diffusion2d/kernels.cu               -> heat2d       (Compute_Laplace2d, Compute_RK)
  SingleGPU/Burgers3d_WENO5/kernels.cu           -> burgers3d    (Compute_dF/dG/dH, Compute_Laplace_Async,
                                                                  Compute_RK)
  SingleGPU/Diffusion3d_Blocking/kernels.cu      -> heat3d_blocking (Compute_Laplace3d_Async, Compute_RK)
(SingleGPU/Burgers3d_WENO5_SharedMem/kernels.cu is not built: its sweeps call __syncthreads
inside `if (I < nx)`, kernels.cu:235-270, which CUDA leaves undefined when a block straddles
the grid's end, as every one of its x tiles does. Its programs still link against the
compatibility library, whose kernels take no such barrier.)
Each is built twice: `<name>.cubin` with nvcc's default flags (FMA contraction on: the reference's
own build, used for timing) and `<name>_nofma.cubin` with -fmad=false (every operation rounded as
written: comparable bit for bit with the FP64 oracle and the library's FP64 path). REAL is double
in all of them (USE_FLOAT false in the reference headers).

The same programs' host tools (SingleGPU/<program>/tools.cpp: initial conditions, result.bin)
are compiled with g++ together with oracle/ref_tools_shim.cpp into host libraries
`libref_tools_<name>.so` (-ffp-contract=off, as the library's host code), for the CPU tests.

Drop-in programs: each program's own main.cpp + tools.cpp (dense and pitched variants) are linked,
unmodified and without their kernels.cu, against the GB300 compatibility library that replaces it
(`refmain_<name>`, once multigpu_advectiondiffusion_gb300/_lib is built). They are linked from
copies staged under oracle/_ref/src/ (git-ignored), so a host of another architecture links
them too (build_mains). The CPU tests check that every symbol resolves; the GPU tests run them.

    python oracle/ref_build.py [--src DIR]

DIR defaults to $ADV_REFERENCE_DIR, else /root/reference (the usual mount point of the reference
checkout; machines without a checkout use the outputs built beside it).
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
UNITS = {
    "heat3d": "SingleGPU/Diffusion3d_baselineCode/kernels.cu",
    "heat2d": "SingleGPU/Diffusion2d/kernels.cu",
    "burgers3d": "SingleGPU/Burgers3d_WENO5/kernels.cu",
    "heat3d_blocking": "SingleGPU/Diffusion3d_Blocking/kernels.cu",
}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
TOOLS = {
    "heat3d": ("SingleGPU/Diffusion3d_baselineCode", "REF_HEAT3D"),
    "heat2d": ("SingleGPU/Diffusion2d", "REF_HEAT2D"),
    "burgers3d": ("SingleGPU/Burgers3d_WENO5", "REF_BURGERS3D"),
}


MAINS = {  # reference program -> the compatibility library that replaces its kernels.cu
    "heat3d": ("SingleGPU/Diffusion3d_baselineCode", "advdiff_compat_heat3d"),
    "heat3d_pitched": ("SingleGPU/Diffusion3d_PitchedMem", "advdiff_compat_heat3d_pitched"),
    "heat2d": ("SingleGPU/Diffusion2d", "advdiff_compat_heat2d"),
    "heat2d_pitched": ("SingleGPU/Diffusion2d_PitchedMem", "advdiff_compat_heat2d_pitched"),
    "burgers3d": ("SingleGPU/Burgers3d_WENO5", "advdiff_compat_burgers3d"),
    "burgers3d_pitched": ("SingleGPU/Burgers3d_WENO5_PitchedMem", "advdiff_compat_burgers3d_pitched"),
    "heat3d_blocking": ("SingleGPU/Diffusion3d_Blocking", "advdiff_compat_heat3d_blocking"),
    "burgers3d_sharedmem": ("SingleGPU/Burgers3d_WENO5_SharedMem", "advdiff_compat_burgers3d_sharedmem"),
}
LIBDIR = HERE.parent / "multigpu_advectiondiffusion_gb300" / "_lib"


def _cuda_include() -> Path:
    nvcc = shutil.which("nvcc")
    inc = Path(nvcc).resolve().parent.parent / "include" if nvcc else Path("/usr/local/cuda/include")
    return inc


def build(src_root: Path) -> list[Path]:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    OUT.mkdir(parents=True, exist_ok=True)
    made = []
    jobs = []
    for name, rel in UNITS.items():
        src = src_root / rel
        if not src.exists():
            raise FileNotFoundError(src)
        for tag, extra in (("", []), ("_nofma", ["-fmad=false"])):
            out = OUT / f"{name}{tag}.cubin"
            if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
                made.append(out)
                continue
            cmd = [nvcc, "-cubin", *ARCH, "-O3", *extra, "-o", str(out), str(src)]
            jobs.append((out, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    shim = HERE / "ref_tools_shim.cpp"
    cxx = shutil.which("g++") or "g++"
    for name, (rel, define) in TOOLS.items():
        src = src_root / rel / "tools.cpp"
        if not src.exists():
            raise FileNotFoundError(src)
        out = OUT / f"libref_tools_{name}.so"
        if out.exists() and out.stat().st_mtime >= max(src.stat().st_mtime, shim.stat().st_mtime):
            made.append(out)
            continue
        cmd = [cxx, "-O2", "-fPIC", "-shared", "-ffp-contract=off", f"-D{define}", "-I", str(src_root / rel),
               "-I", str(_cuda_include()), "-w", "-o", str(out), str(shim), str(src), "-lm"]
        jobs.append((out, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    stage_sources(src_root)
    jobs += _main_jobs(made)
    for out, p in jobs:
        log, _ = p.communicate()
        if p.returncode != 0:
            if out.suffix == ".cubin":
                raise RuntimeError(f"reference build failed for {out.name}:\n{log}")
            # host tools and linked mains are checks of their own: their tests skip without them
            print(f"warning: {out.name} not built:\n{log[-2000:]}", file=sys.stderr)
            continue
        made.append(out)
    return made


def stage_sources(src_root: Path) -> None:
    """Copies each linked program's own main.cpp, tools.cpp and headers, unmodified, into
    oracle/_ref/src/<name>/ (git-ignored like the rest of oracle/_ref, never committed). The GPU
    hosts are another architecture and have no reference checkout: build() links the programs
    there from these copies."""
    for name, (rel, _) in MAINS.items():
        d = src_root / rel
        if not (d / "main.cpp").exists():
            continue
        dst = OUT / "src" / name
        dst.mkdir(parents=True, exist_ok=True)
        for f in [d / "main.cpp", d / "tools.cpp", *sorted(d.glob("*.h"))]:
            t = dst / f.name
            if not t.exists() or t.stat().st_mtime < f.stat().st_mtime:
                shutil.copy2(f, t)


def _main_jobs(made: list) -> list:
    """Compile jobs linking each staged program against the compatibility library that replaces
    its kernels.cu (refmain_<name>); up-to-date outputs go straight to `made`."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    jobs = []
    for name, (_, compat) in MAINS.items():
        lib = LIBDIR / f"lib{compat}.so"
        stage = OUT / "src" / name
        srcs = [stage / "main.cpp", stage / "tools.cpp"]
        if not lib.exists() or not all(x.exists() for x in srcs):
            continue
        out = OUT / f"refmain_{name}"
        if out.exists() and out.stat().st_mtime >= max(x.stat().st_mtime for x in srcs + [lib]):
            made.append(out)
            continue
        rpath = "-rpath,$ORIGIN/../../multigpu_advectiondiffusion_gb300/_lib"
        # -ffp-contract=off: the programs' host arithmetic (their initial conditions) rounds as written
        # on every host, as the oracle and the library's host code do; g++ would otherwise fuse
        # multiply-adds on Arm hosts (FMA is in the base ISA there, not on x86-64)
        cmd = [nvcc, *ARCH, "-O3", "-w", "-Xcompiler", "-ffp-contract=off", "-o", str(out), *map(str, srcs),
               "-L", str(LIBDIR), f"-l{compat}", "-ladvdiff", "-Xlinker", rpath]
        jobs.append((out, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    return jobs


def build_mains() -> list[Path]:
    """Links the staged reference programs on this host (no reference checkout needed)."""
    made: list[Path] = []
    for out, p in _main_jobs(made):
        log, _ = p.communicate()
        if p.returncode != 0:
            print(f"warning: {out.name} not built:\n{log[-2000:]}", file=sys.stderr)
            continue
        made.append(out)
    return made


def reference_dir() -> Path | None:
    """The reference checkout to build from: $ADV_REFERENCE_DIR, else /root/reference; None if absent."""
    p = Path(os.environ.get("ADV_REFERENCE_DIR", "/root/reference"))
    return p if p.is_dir() else None


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=str(reference_dir() or "/root/reference"))
    a = ap.parse_args(argv)
    for p in build(Path(a.src)):
        print(p.relative_to(HERE.parent))


if __name__ == "__main__":
    main(sys.argv[1:])
