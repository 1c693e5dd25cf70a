"""The library against the reference's own host code (CPU only), built from the reference
sources by oracle/ref_build.py into oracle/_ref/:
* row a11: the initial conditions and the result.bin writer of
  SingleGPU/{Diffusion3d_baselineCode,Diffusion2d,Burgers3d_WENO5}/tools.cpp equal the library's
  adv_ic_*_ref and adv_write_result_bin bit for bit;
* the drop-in link: each program's own main.cpp + tools.cpp, dense and pitched, links unmodified
  against the compatibility library that replaces its kernels.cu.
Skipped where the reference sources were not available at build time."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N

REF = Path(__file__).resolve().parent.parent / "oracle" / "_ref"


def _tools(name):
    so = REF / f"libref_tools_{name}.so"
    if not so.exists():
        pytest.skip(f"{so.name} not built (needs the reference sources at build time)")
    lib = C.CDLL(str(so))
    lib.ref_init.argtypes = [C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_uint, C.c_uint, C.c_uint]
    lib.ref_save_binary.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint]
    return lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.parametrize("shape,h", [((21, 19, 17), (0.5, 0.55, 0.6)), ((40, 33, 26), (10 / 39, 10 / 32, 10 / 25))])
def test_heat3d_initial_condition_equals_the_reference(native, shape, h):
    ref = _tools("heat3d")
    nx, ny, nz = shape
    want = np.full(nx * ny * nz, np.nan)
    ref.ref_init(3, want.ctypes.data, *h, nx, ny, nz)
    got = np.empty_like(want)
    assert native.adv_ic_heat_ref(3, nx, ny, nz, *h, _dp(got)) == N.ADV_OK
    assert np.array_equal(got, want)


def test_heat2d_initial_condition_equals_the_reference(native):
    ref = _tools("heat2d")
    nx, ny = 51, 47
    h = (10 / 50, 10 / 46)
    want = np.full(nx * ny, np.nan)
    ref.ref_init(3, want.ctypes.data, h[0], h[1], 0.0, nx, ny, 1)
    got = np.empty_like(want)
    assert native.adv_ic_heat_ref(2, nx, ny, 1, h[0], h[1], 0.0, _dp(got)) == N.ADV_OK
    assert np.array_equal(got, want)


def test_burgers_initial_condition_equals_the_reference(native):
    ref = _tools("burgers3d")
    nx, ny, nz = 24, 22, 20
    h = (2 / 23, 2 / 21, 2 / 19)
    want = np.full(nx * ny * nz, np.nan)
    ref.ref_init(3, want.ctypes.data, *h, nx, ny, nz)
    got = np.empty_like(want)
    assert native.adv_ic_burgers_ref(nx, ny, nz, *h, _dp(got)) == N.ADV_OK
    assert np.array_equal(got, want)


@pytest.mark.parametrize("name,shape", [("heat3d", (9, 8, 7)), ("heat2d", (13, 11, 1)), ("burgers3d", (6, 5, 4))])
def test_result_bin_equals_the_reference_writer(native, tmp_path, monkeypatch, name, shape):
    ref = _tools(name)
    u = np.random.default_rng(3).standard_normal(int(np.prod(shape))) * 1e3
    monkeypatch.chdir(tmp_path)
    ref.ref_save_binary(u.ctypes.data, *shape)  # writes result.bin in the working directory
    ours = tmp_path / "ours.bin"
    assert native.adv_write_result_bin(str(ours).encode(), N.ADV_F64, u.ctypes.data, u.size) == N.ADV_OK
    assert (tmp_path / "result.bin").read_bytes() == ours.read_bytes()


@pytest.mark.parametrize("name,lib,wrappers", [
    ("heat3d", "advdiff_compat_heat3d", {"CopyToConstantMemory", "Call_Lu3d", "Call_RK3d"}),
    ("heat3d_pitched", "advdiff_compat_heat3d_pitched", {"CopyToConstantMemory", "Call_Lu3d", "Call_RK3d"}),
    ("heat2d", "advdiff_compat_heat2d", {"CopyToConstantMemory", "Call_Lu2d", "Call_RK2d"}),
    ("heat2d_pitched", "advdiff_compat_heat2d_pitched", {"CopyToConstantMemory", "Call_Lu2d", "Call_RK2d"}),
    ("burgers3d", "advdiff_compat_burgers3d",
     {"CopyToConstantMemory", "Call_Adv_x", "Call_Adv_y", "Call_Adv_z", "Call_Diff_", "Call_sspRK"}),
    ("burgers3d_pitched", "advdiff_compat_burgers3d_pitched",
     {"CopyToConstantMemory", "Call_Adv_x", "Call_Adv_y", "Call_Adv_z", "Call_Diff_", "Call_sspRK"}),
    ("heat3d_blocking", "advdiff_compat_heat3d_blocking", {"CopyToConstantMemory", "Call_Lu3d", "Call_RK3d"}),
    ("burgers3d_sharedmem", "advdiff_compat_burgers3d_sharedmem",
     {"CopyToConstantMemory", "Call_Adv_x", "Call_Adv_y", "Call_Adv_z", "Call_Diff_", "Call_sspRK"}),
])
def test_reference_main_links_against_the_compat_library(native, name, lib, wrappers):
    """The reference program's own main.cpp + tools.cpp, unmodified and without its kernels.cu,
    linked against the compatibility library (oracle/ref_build.py): every symbol resolves, and
    the kernel wrappers it calls come from the GB300 library."""
    import subprocess
    exe = REF / f"refmain_{name}"
    if not exe.exists():
        pytest.skip(f"{exe.name} not built (needs the reference sources at build time)")
    r = subprocess.run(["ldd", "-r", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and "undefined symbol" not in r.stdout + r.stderr and "not found" not in r.stdout
    undefined = subprocess.run(["nm", "-D", "--undefined-only", str(exe)], capture_output=True, text=True,
                               check=True).stdout
    assert wrappers <= {l.split()[-1] for l in undefined.splitlines() if l.strip()}
    exported = subprocess.run(["nm", "-D", "--defined-only", str(N.LIBDIR / f"lib{lib}.so")], capture_output=True,
                              text=True, check=True).stdout
    assert wrappers <= {l.split()[-1] for l in exported.splitlines() if " T " in l}
