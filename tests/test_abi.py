"""The C-ABI libraries load and export every declared symbol; host-side entry points agree
with the oracle. No GPU calls."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N

ROOT = Path(__file__).resolve().parent.parent


def _declared(header: Path, define_pitched: bool = False) -> set[str]:
    txt = header.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt, flags=re.M))
    return {n for n in names if n not in {"defined", "if", "ifdef", "ifndef"}}


def _exports(so: Path) -> set[str]:
    out = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True, check=True).stdout
    return {l.split()[-1] for l in out.splitlines() if " T " in l}


def test_native_exports_every_declared_symbol(native):
    exp = _exports(N.lib_path())
    for h in ("advdiff.h", "advdiff_ref_ops.h"):
        missing = _declared(ROOT / "include" / h) - exp
        assert not missing, (h, missing)
    for name, _, _ in N.SIGNATURES:
        assert name in exp


@pytest.mark.parametrize("lib,header,names", [
    ("libadvdiff_compat_heat3d.so", "advdiff_compat_heat3d.h", {"CopyToConstantMemory", "Call_Lu3d", "Call_RK3d"}),
    ("libadvdiff_compat_heat2d.so", "advdiff_compat_heat2d.h", {"CopyToConstantMemory", "Call_Lu2d", "Call_RK2d"}),
    ("libadvdiff_compat_burgers3d.so", "advdiff_compat_burgers3d.h",
     {"CopyToConstantMemory", "Call_Adv_x", "Call_Adv_y", "Call_Adv_z", "Call_Diff_", "Call_sspRK"}),
])
@pytest.mark.parametrize("pitched", [False, True])
def test_compat_exports_reference_names(native, lib, header, names, pitched):
    so = N.LIBDIR / (lib.replace(".so", "_pitched.so") if pitched else lib)
    C.CDLL(str(so))
    exp = _exports(so)
    assert names | {"adv_compat_last_status"} <= exp
    assert _declared(ROOT / "include" / header) <= exp


@pytest.mark.parametrize("lib,header,names", [
    ("libadvdiff_compat_heat3d_blocking.so", "advdiff_compat_heat3d.h",
     {"CopyToConstantMemory", "Call_Lu3d", "Call_RK3d"}),
    ("libadvdiff_compat_burgers3d_sharedmem.so", "advdiff_compat_burgers3d.h",
     {"CopyToConstantMemory", "Call_Adv_x", "Call_Adv_y", "Call_Adv_z", "Call_Diff_", "Call_sspRK"}),
])
def test_compat_variant_libraries_export_reference_names(native, lib, header, names):
    """The z-blocked heat and shared-memory Burgers programs' libraries (pitched signatures)."""
    so = N.LIBDIR / lib
    C.CDLL(str(so))
    exp = _exports(so)
    assert names | {"adv_compat_last_status"} <= exp
    assert _declared(ROOT / "include" / header) <= exp


def test_ref_variant_ops_reject_bad_arguments_without_gpu(native):
    buf = C.c_void_p(64)
    box = (C.c_int32 * 6)(3, 9, 3, 9, 3, 10)
    # k1 = nz - 1 would read a plane past the grid (the O4 stencil needs k + 2 < nz)
    bad = (C.c_int32 * 6)(3, 9, 3, 9, 3, 11)
    assert native.adv_ref_laplace_box(N.ADV_F64, 3, 4, bad, 0, 1, 12, 12, 12, 12, 1.0, 1.0, 1.0, buf, buf,
                                      None) == N.ADV_ERR_INVALID_ARG
    assert b"margin" in native.adv_last_error_string()
    assert native.adv_ref_laplace_box(N.ADV_F64, 3, 4, None, 0, 1, 12, 12, 12, 12, 1.0, 1.0, 1.0, buf, buf,
                                      None) == N.ADV_ERR_INVALID_ARG
    assert native.adv_ref_laplace_box(N.ADV_F64, 3, 3, box, 0, 1, 12, 12, 12, 12, 1.0, 1.0, 1.0, buf, buf,
                                      None) == N.ADV_ERR_INVALID_ARG
    assert native.adv_ref_laplace_box(N.ADV_F64, 3, 4, box, 0, 2, 12, 12, 12, 12, 1.0, 1.0, 1.0, buf, buf,
                                      None) == N.ADV_ERR_INVALID_ARG
    assert native.adv_ref_burgers_sweep_all(N.ADV_F64, 3, N.ADV_WENO5_Z, 12, 12, 12, 12, 0.1, buf, buf,
                                            None) == N.ADV_ERR_INVALID_ARG
    assert native.adv_ref_burgers_sweep_all(N.ADV_F64, 0, N.ADV_WENO5_Z, 12, 12, 12, 12, 0.0, buf, buf,
                                            None) == N.ADV_ERR_INVALID_ARG
    assert native.adv_ref_burgers_sweep_all(N.ADV_F64, 0, N.ADV_WENO5_Z, 8, 12, 12, 12, 0.1, buf, buf,
                                            None) == N.ADV_ERR_INVALID_ARG  # pitch < nx


def test_abi_version_and_strings(native):
    assert native.adv_abi_version() == 3
    assert native.adv_status_string(N.ADV_ERR_TIMEOUT) == b"ADV_ERR_TIMEOUT"


def test_invalid_descriptors_rejected_without_gpu(native):
    nb = C.c_size_t(0)
    bad = N.HeatDesc(4, 8, 8, 8, N.ADV_F32, 2, 1, 1, 1.0, 1.0, 1.0, 0.1)
    assert native.adv_heat_workspace_bytes(C.byref(bad), N.ADV_EULER, C.byref(nb)) == N.ADV_ERR_INVALID_ARG
    assert b"ndim" in native.adv_last_error_string()
    thin = N.HeatDesc(3, 8, 8, 8, N.ADV_F32, 4, 1, 0, 1.0, 1.0, 1.0, 0.1)  # frozen < radius
    assert native.adv_heat_workspace_bytes(C.byref(thin), N.ADV_EULER, C.byref(nb)) == N.ADV_ERR_INVALID_ARG
    empty = N.HeatDesc(3, 0, 8, 8, N.ADV_F32, 2, 1, 0, 1.0, 1.0, 1.0, 0.1)
    assert native.adv_heat_workspace_bytes(C.byref(empty), N.ADV_EULER, C.byref(nb)) == N.ADV_ERR_INVALID_ARG
    ok = N.HeatDesc(3, 9, 8, 7, N.ADV_F64, 2, 1, 1, 1.0, 1.0, 1.0, 0.1)
    assert native.adv_heat_workspace_bytes(C.byref(ok), N.ADV_SSPRK3, C.byref(nb)) == N.ADV_OK
    assert nb.value == 2 * ((9 * 8 * 7 * 8 + 255) // 256 * 256)
    bd = N.BurgersDesc(4, 8, 8, N.ADV_F32, 1, 1, N.ADV_BC_PERIODIC, 0, 0, 0, 1.0, 1.0, 1.0, 0, 0, 0)
    assert native.adv_burgers_workspace_bytes(C.byref(bd), C.byref(nb)) == N.ADV_ERR_INVALID_ARG


def test_launching_entry_points_reject_bad_arguments_without_gpu(native):
    """Each entry point that launches work opens its NVTX range, then validates its arguments
    before any CUDA call: with no GPU the bad request still comes back as ADV_ERR_INVALID_ARG."""
    bad = N.HeatDesc(4, 8, 8, 8, N.ADV_F32, 2, 1, 1, 1.0, 1.0, 1.0, 0.1)
    assert native.adv_heat_run(C.byref(bad), N.ADV_EULER, 4, None, None, None) == N.ADV_ERR_INVALID_ARG
    assert native.adv_heat_run_noalloc(C.byref(bad), N.ADV_EULER, 4, None, None) == N.ADV_ERR_INVALID_ARG
    ok = N.HeatDesc(3, 16, 16, 16, N.ADV_F32, 2, 1, 1, 1.0, 1.0, 1.0, 0.1)
    buf = C.c_void_p(16)
    # the failure-path test launch checks its plane and wait limit before any CUDA call
    assert native.adv_test_heat_stage_withheld(C.byref(ok), 1, buf, buf, C.c_void_p(32), 16, 10 ** 6,
                                               None) == N.ADV_ERR_INVALID_ARG
    assert b"withheld plane" in native.adv_last_error_string()
    assert native.adv_test_heat_stage_withheld(C.byref(ok), 1, buf, buf, C.c_void_p(32), 3, 10,
                                               None) == N.ADV_ERR_INVALID_ARG
    assert b"wait limit" in native.adv_last_error_string()
    bd = N.BurgersDesc(4, 8, 8, N.ADV_F32, 1, 1, N.ADV_BC_PERIODIC, 0, 0, 0, 1.0, 1.0, 1.0, 0, 0, 0)
    t, s = C.c_double(0.0), C.c_int64(0)
    assert native.adv_burgers_run(C.byref(bd), None, None, 1.0, 0.5, N.ADV_DT_FIXED, 0.0, 10, C.byref(t),
                                  C.byref(s), None) == N.ADV_ERR_INVALID_ARG
    assert b"at least 6 cells" in native.adv_last_error_string()
    out = C.c_double(0.0)
    assert native.adv_max_abs(99, None, 4, C.byref(out), None) == N.ADV_ERR_INVALID_ARG
    assert native.adv_ref_laplace(99, 3, 2, 1, 0, 8, 8, 8, 8, 1.0, 1.0, 1.0, None, None, None) == N.ADV_ERR_INVALID_ARG
    # repeated calls: the ranges push and pop in pairs, nothing accumulates
    for _ in range(1000):
        assert native.adv_max_abs(99, None, 4, C.byref(out), None) == N.ADV_ERR_INVALID_ARG


def test_ensemble_argument_checks_without_gpu(native):
    out = C.c_void_p(None)
    assert native.adv_ensemble_create(None, 0, N.ADV_EULER, None, 0, C.byref(out)) == N.ADV_ERR_INVALID_ARG
    assert b"no members" in native.adv_last_error_string()
    hm = (N.HeatMember * 1)()
    assert native.adv_ensemble_create(hm, 1, 7, None, 0, C.byref(out)) == N.ADV_ERR_INVALID_ARG
    assert b"time scheme" in native.adv_last_error_string()
    assert native.adv_ensemble_create(None, 2, N.ADV_EULER, None, 0, C.byref(out)) == N.ADV_ERR_INVALID_ARG
    assert out.value is None
    assert native.adv_ensemble_run(None, 1, 0, None) == N.ADV_ERR_INVALID_ARG
    assert native.adv_ensemble_destroy(None) == N.ADV_OK


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def test_host_initial_conditions_equal_oracle(native, oracle):
    u = np.empty(33 * 31 * 29)
    assert native.adv_ic_heat3d_blobs(33, 31, 29, 2, 8, _dp(u)) == 0
    np.testing.assert_array_equal(u, oracle.ic_heat3d_blobs(33, 31, 29, 2, 8))
    v = np.empty(40 * 36)
    assert native.adv_ic_heat2d_gauss_noise(40, 36, 1, 1e-3, _dp(v)) == 0
    np.testing.assert_array_equal(v, oracle.ic_heat2d_gauss_noise(40, 36, 1, 1e-3))
    w = np.empty(20 * 18 * 16)
    assert native.adv_ic_burgers_fourier(20, 18, 16, 2.0, 3, 16, 0.1, _dp(w)) == 0
    np.testing.assert_array_equal(w, oracle.ic_burgers_fourier(20, 18, 16, 2.0, 3, 16, 0.1))
    r = np.empty(21 * 19 * 17)
    assert native.adv_ic_heat_ref(3, 21, 19, 17, 0.5, 0.55, 0.6, _dp(r)) == 0
    np.testing.assert_array_equal(r, oracle.ic_heat_ref(3, 21, 19, 17, 0.5, 0.55, 0.6))
    b = np.empty(12 * 11 * 10)
    assert native.adv_ic_burgers_ref(12, 11, 10, 0.2, 0.2, 0.2, _dp(b)) == 0
    np.testing.assert_array_equal(b, oracle.ic_burgers_ref(12, 11, 10, 0.2, 0.2, 0.2))


def test_result_bin_layout(native, tmp_path):
    """result.bin: float32, x fastest, no header (SingleGPU/Diffusion3d_baselineCode/tools.cpp:59-87)."""
    u = np.arange(4 * 3 * 2, dtype=np.float64) / 7.0
    p = tmp_path / "result.bin"
    assert native.adv_write_result_bin(str(p).encode(), N.ADV_F64, u.ctypes.data, u.size) == 0
    got = np.fromfile(p, dtype=np.float32)
    np.testing.assert_array_equal(got, u.astype(np.float32))
    assert p.stat().st_size == 4 * u.size


def test_drivers_print_usage_without_gpu(native):
    for drv in ("heat2d", "heat3d", "burgers3d", "burgers2d"):
        r = subprocess.run([str(N.LIBDIR / drv)], capture_output=True, text=True)
        assert r.returncode == 1 and "Usage" in r.stdout


@pytest.mark.parametrize("header", ["advdiff.h", "advdiff_ref_ops.h", "advdiff_compat_heat2d.h",
                                    "advdiff_compat_heat3d.h", "advdiff_compat_burgers3d.h"])
@pytest.mark.parametrize("lang", ["c99", "c++17"])
def test_headers_compile_as_c_and_cpp(tmp_path, header, lang):
    """The boundary headers are plain C (what a cgo / FFI / C host includes) and valid C++; the
    native ones need no CUDA header, the compatibility ones include cuda_runtime.h for dim3."""
    import shutil
    cc = shutil.which("gcc" if lang == "c99" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    src = tmp_path / ("t.c" if lang == "c99" else "t.cpp")
    src.write_text(f'#include "{header}"\nint main(void) {{ return 0; }}\n')
    cmd = [cc, f"-std={lang}", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include")]
    if "compat" in header:
        nvcc = shutil.which("nvcc")
        cuda_inc = Path(nvcc).resolve().parent.parent / "include" if nvcc else Path("/usr/local/cuda/include")
        if not (cuda_inc / "cuda_runtime.h").exists():
            pytest.skip("no CUDA toolkit headers")
        cmd += ["-I", str(cuda_inc)]
    else:
        cmd += ["-pedantic"]
    r = subprocess.run(cmd + [str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_c_host_links_and_calls_the_library(native, tmp_path):
    """A plain C99 program links libadvdiff.so and uses its host-side entry points (no GPU):
    the seeded initial condition, result.bin written and read back, status strings."""
    import shutil
    if shutil.which("gcc") is None:
        pytest.skip("no host compiler")
    src = tmp_path / "host.c"
    src.write_text(r'''
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "advdiff.h"
int main(int argc, char** argv) {
  enum { NX = 9, NY = 8, NZ = 7, N = NX * NY * NZ };
  double u[N], back[N];
  if (adv_abi_version() != ADV_ABI_VERSION) return 2;
  if (adv_ic_heat_ref(3, NX, NY, NZ, 0.5, 0.5, 0.5, u) != ADV_OK) return 3;
  if (adv_write_result_bin(argv[1], ADV_F64, u, N) != ADV_OK) return 4;
  if (adv_read_result_bin(argv[1], N, back) != ADV_OK) return 5;
  for (int i = 0; i < N; ++i)
    if (back[i] != (double)(float)u[i]) return 6;
  if (adv_read_result_bin(argv[1], N + 1, back) != ADV_ERR_INVALID_ARG) return 7;
  if (strcmp(adv_status_string(ADV_ERR_CFL), "ADV_ERR_CFL") != 0) return 8;
  printf("ok %s\n", adv_last_error_string());
  return argc == 2 ? 0 : 9;
}
''')
    exe = tmp_path / "host"
    lib = N.lib_path()
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                        "-L", str(lib.parent), "-ladvdiff", f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe), str(tmp_path / "result.bin")], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, (run.returncode, run.stdout, run.stderr)
    assert run.stdout.startswith("ok")


def _prototypes(header: Path) -> dict[str, tuple[str, list[str]]]:
    txt = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    txt = re.sub(r"^\s*#.*$", "", txt, flags=re.M)
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(adv_\w+)\s*\(([^()]*)\)\s*;", txt):
        params = [p.strip() for p in m.group(3).split(",")]
        if params == ["void"] or params == [""]:
            params = []
        out[m.group(2)] = (m.group(1).strip(), params)
    return out


def _ctype_ok(decl: str, ct) -> bool:
    """Does the ctypes type `ct` pass a C parameter / return value declared as `decl`?"""
    decl = re.sub(r"\b(const|struct)\b", "", decl)
    if "*" in decl:
        base = decl.split("*")[0].split()[0]
        structs = {"adv_heat_desc": N.HeatDesc, "adv_burgers_desc": N.BurgersDesc, "adv_heatk_desc": N.HeatKDesc,
                   "adv_weno7_desc": N.Weno7Desc,
                   "adv_heat_member": N.HeatMember, "adv_burgers_member": N.BurgersMember,
                   "adv_tune_result": N.TuneResult, "adv_checkpoint_header": N.CheckpointHeader}
        if base == "char":
            return ct is C.c_char_p
        if decl.count("*") == 2:
            return ct is C.POINTER(C.c_void_p)
        if base in structs:
            return ct is C.POINTER(structs[base])
        if base == "adv_ensemble":
            return ct is C.c_void_p
        if base == "void":
            return ct is C.c_void_p
        scalar = {"double": C.c_double, "int64_t": C.c_int64, "size_t": C.c_size_t, "int": C.c_int,
                  "int32_t": C.c_int32}[base]
        return ct is C.POINTER(scalar) or ct is C.c_void_p
    base = decl.split()[0]
    scalar = {"double": C.c_double, "int64_t": C.c_int64, "size_t": C.c_size_t, "int": C.c_int, "int32_t": C.c_int32,
              "uint32_t": C.c_uint32, "uint64_t": C.c_uint64, "adv_status": C.c_int}
    return ct is scalar[base]


def test_ctypes_signatures_match_the_header_prototypes():
    """Every entry of _native.SIGNATURES passes the same number and kinds of arguments as the C
    prototype it binds, and every declared entry point is bound."""
    protos = {**_prototypes(ROOT / "include" / "advdiff.h"), **_prototypes(ROOT / "include" / "advdiff_ref_ops.h")}
    bound = {name: (res, args) for name, res, args in N.SIGNATURES}
    assert set(protos) <= set(bound), set(protos) - set(bound)
    for name, (ret, params) in protos.items():
        res, args = bound[name]
        assert len(args) == len(params), (name, params)
        assert _ctype_ok(ret, res), (name, ret, res)
        for p, a in zip(params, args):
            typ = re.sub(r"\s*\b\w+$", "", p) if not p.endswith("*") else p  # drop the parameter name
            assert _ctype_ok(typ, a), (name, p, a)


def test_ctypes_structures_match_the_c_layout(tmp_path):
    """sizeof and every field offset of the descriptor / member / result structs, as a C compiler
    lays them out, equal the ctypes Structures the Python host passes."""
    import shutil
    if shutil.which("gcc") is None:
        pytest.skip("no host compiler")
    structs = {"adv_heat_desc": N.HeatDesc, "adv_burgers_desc": N.BurgersDesc, "adv_heatk_desc": N.HeatKDesc,
               "adv_weno7_desc": N.Weno7Desc,
               "adv_heat_member": N.HeatMember, "adv_burgers_member": N.BurgersMember,
               "adv_tune_result": N.TuneResult, "adv_checkpoint_header": N.CheckpointHeader}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "advdiff.h"', "int main(void) {"]
    want = []
    for cname, py in structs.items():
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        want.append(C.sizeof(py))
        for fname, _ in py._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {fname}));')
            want.append(getattr(py, fname).offset)
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == want


def test_checked_build_exports_the_same_symbols_and_says_so(native):
    """libadvdiff_checked.so (ADV_BOUNDS_CHECK) exports every declared symbol; adv_bounds_checked()
    is 1 there and 0 in the normal build (callable without a GPU)."""
    so = N.LIBDIR / "libadvdiff_checked.so"
    exp = _exports(so)
    for h in ("advdiff.h", "advdiff_ref_ops.h"):
        assert _declared(ROOT / "include" / h) <= exp
    checked = C.CDLL(str(so))
    assert checked.adv_bounds_checked() == 1
    assert native.adv_bounds_checked() == 0
    assert native.adv_status_string(N.ADV_ERR_BOUNDS) == b"ADV_ERR_BOUNDS"
