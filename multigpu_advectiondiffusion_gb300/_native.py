"""ctypes bindings of the native C ABI (include/advdiff.h, include/advdiff_ref_ops.h).

The CUDA library is the only compute path: if ``libadvdiff.so`` is missing this module raises
at import time instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIBDIR = Path(__file__).resolve().parent / "_lib"

ADV_OK, ADV_ERR_INVALID_ARG, ADV_ERR_CUDA, ADV_ERR_TIMEOUT = 0, 1, 2, 3
ADV_ERR_NONFINITE, ADV_ERR_CFL, ADV_ERR_UNSUPPORTED, ADV_ERR_ALLOC, ADV_ERR_BOUNDS = 4, 5, 6, 7, 8
ADV_F32, ADV_F64 = 0, 1
ADV_EULER, ADV_SSPRK3 = 0, 1
ADV_WENO5_JS, ADV_WENO5_Z = 0, 1
ADV_LF_LOCAL, ADV_LF_GLOBAL = 0, 1
ADV_BC_FROZEN, ADV_BC_PERIODIC = 0, 1
ADV_DIV_F32, ADV_DIV_F64, ADV_DIV_FAST = 0, 1, 2
ADV_DT_FIXED, ADV_DT_MAXU = 0, 1
ADV_ENSEMBLE_DIRECT = 1
ADV_HEATK_LAST_INTERVAL_IN_WORK = 1
ADV_BURGERS_LAST_INTERVAL_IN_WORK = 1


class HeatDesc(C.Structure):
    """adv_heat_desc (include/advdiff.h)."""
    _fields_ = [("ndim", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("dtype", C.c_int32), ("order", C.c_int32), ("frozen", C.c_int32), ("zero_boundary", C.c_int32),
                ("kx", C.c_double), ("ky", C.c_double), ("kz", C.c_double), ("dt", C.c_double),
                ("contract", C.c_int32), ("pad0", C.c_int32)]


class BurgersDesc(C.Structure):
    """adv_burgers_desc (include/advdiff.h)."""
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("dtype", C.c_int32),
                ("weno", C.c_int32), ("lf", C.c_int32), ("bc", C.c_int32), ("div", C.c_int32),
                ("bug_b2", C.c_int32), ("pad0", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("kx", C.c_double), ("ky", C.c_double), ("kz", C.c_double)]


class Weno7Desc(C.Structure):
    """adv_weno7_desc (include/advdiff.h)."""
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("dtype", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double)]


class HeatKDesc(C.Structure):
    """adv_heatk_desc (include/advdiff.h)."""
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("dtype", C.c_int32),
                ("zero_boundary", C.c_int32), ("pad0", C.c_int32),
                ("cx", C.c_double), ("cy", C.c_double), ("cz", C.c_double)]


class TuneResult(C.Structure):
    """adv_tune_result (include/advdiff.h)."""
    _fields_ = [("kind", C.c_int32), ("param_a", C.c_int32), ("param_b", C.c_int32), ("candidates", C.c_int32),
                ("best_us", C.c_double), ("default_us", C.c_double)]


class CheckpointHeader(C.Structure):
    """adv_checkpoint_header (include/advdiff.h)."""
    _fields_ = [("version", C.c_int32), ("dtype", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32),
                ("nz", C.c_int32), ("pad0", C.c_int32), ("step", C.c_int64), ("t", C.c_double),
                ("payload_bytes", C.c_uint64), ("payload_crc32", C.c_uint32), ("pad1", C.c_uint32)]


class HeatMember(C.Structure):
    """adv_heat_member (include/advdiff.h)."""
    _fields_ = [("desc", HeatDesc), ("u", C.c_void_p), ("work", C.c_void_p)]


class BurgersMember(C.Structure):
    """adv_burgers_member (include/advdiff.h)."""
    _fields_ = [("desc", BurgersDesc), ("u", C.c_void_p), ("work", C.c_void_p), ("tEnd", C.c_double),
                ("cfl", C.c_double), ("dt_rule", C.c_int32), ("pad0", C.c_int32), ("C", C.c_double),
                ("max_steps", C.c_int64)]


# (name, restype, argtypes) for every symbol declared in include/advdiff.h and advdiff_ref_ops.h
_VP, _I, _I64, _D = C.c_void_p, C.c_int, C.c_int64, C.c_double
_PD = C.POINTER(C.c_double)
SIGNATURES = [
    ("adv_heat_stage", _I, [C.POINTER(HeatDesc), _I, _VP, _VP, _VP, _VP]),
    ("adv_heat_workspace_bytes", _I, [C.POINTER(HeatDesc), _I, C.POINTER(C.c_size_t)]),
    ("adv_heat_run", _I, [C.POINTER(HeatDesc), _I, _I64, _VP, _VP, _VP]),
    ("adv_heat_run_noalloc", _I, [C.POINTER(HeatDesc), _I, _I64, _VP, _VP]),
    ("adv_device_status", _I, [_VP]),
    ("adv_bounds_checked", _I, []),
    ("adv_test_heat_stage_withheld", _I, [C.POINTER(HeatDesc), _I, _VP, _VP, _VP, _I, C.c_uint64, _VP]),
    ("adv_burgers_stage", _I, [C.POINTER(BurgersDesc), _I, _VP, _VP, _VP, _D, _D, _VP, _VP]),
    ("adv_burgers_workspace_bytes", _I, [C.POINTER(BurgersDesc), C.POINTER(C.c_size_t)]),
    ("adv_burgers_run", _I, [C.POINTER(BurgersDesc), _VP, _VP, _D, _D, _I, _D, _I64, _PD,
                             C.POINTER(C.c_int64), _VP]),
    ("adv_weno7_workspace_bytes", _I, [C.POINTER(Weno7Desc), C.POINTER(C.c_size_t)]),
    ("adv_weno7_rhs", _I, [C.POINTER(Weno7Desc), _VP, _VP, _VP, _VP]),
    ("adv_weno7_run", _I, [C.POINTER(Weno7Desc), _VP, _VP, _D, _D, _I64, _PD, C.POINTER(C.c_int64), _VP]),
    ("adv_heatk_step", _I, [C.POINTER(HeatKDesc), _VP, _VP, _VP, _VP]),
    ("adv_heatk_adjoint_step", _I, [C.POINTER(HeatKDesc), _VP, _VP, _VP, _VP, _VP, _VP]),
    ("adv_heatk_checkpoint_bytes", _I, [C.POINTER(HeatKDesc), _I64, _I64, C.POINTER(C.c_size_t),
                                        C.POINTER(C.c_size_t)]),
    ("adv_heatk_forward", _I, [C.POINTER(HeatKDesc), _VP, _VP, _I64, _I64, _VP, _VP, _VP]),
    ("adv_heatk_backward", _I, [C.POINTER(HeatKDesc), _VP, _I64, _I64, _VP, _VP, _VP, _VP, _I, _VP]),
    ("adv_burgers_adjoint_step", _I, [C.POINTER(BurgersDesc), _VP, _VP, _VP, _D, _VP, _VP, _VP]),
    ("adv_burgers_checkpoint_bytes", _I, [C.POINTER(BurgersDesc), _I64, _I64, C.POINTER(C.c_size_t),
                                          C.POINTER(C.c_size_t)]),
    ("adv_burgers_forward", _I, [C.POINTER(BurgersDesc), _VP, _D, _I64, _I64, _VP, _VP, _VP]),
    ("adv_burgers_backward", _I, [C.POINTER(BurgersDesc), _D, _I64, _I64, _VP, _VP, _VP, _I, _VP]),
    ("adv_ensemble_create", _I, [C.POINTER(HeatMember), _I, _I, C.POINTER(BurgersMember), _I,
                                 C.POINTER(_VP)]),
    ("adv_ensemble_run", _I, [_VP, _I64, _I, _VP]),
    ("adv_ensemble_burgers_result", _I, [_VP, _I, _PD, C.POINTER(C.c_int64)]),
    ("adv_ensemble_shape", _I, [_VP, C.POINTER(C.c_int64), C.POINTER(C.c_int), C.POINTER(C.c_int64),
                                C.POINTER(C.c_int)]),
    ("adv_ensemble_destroy", _I, [_VP]),
    ("adv_autotune_heat", _I, [C.POINTER(HeatDesc), _VP, _VP, C.POINTER(TuneResult)]),
    ("adv_autotune_burgers", _I, [C.POINTER(BurgersDesc), _VP, _VP, C.POINTER(TuneResult)]),
    ("adv_autotune_heatk", _I, [C.POINTER(HeatKDesc), _VP, _VP, _VP, C.POINTER(TuneResult), C.POINTER(TuneResult)]),
    ("adv_autotune_clear", _I, []),
    ("adv_autotune_export", _I, [C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    ("adv_autotune_import", _I, [C.c_char_p]),
    ("adv_burgers_resume", _I, [C.POINTER(BurgersDesc), _VP, _VP, _D, _I64, _D, _D, _I, _D, _I64, _PD,
                                C.POINTER(C.c_int64), _VP]),
    ("adv_max_abs", _I, [_I, _VP, _I64, _PD, _VP]),
    ("adv_ic_heat_ref", _I, [_I, _I, _I, _I, _D, _D, _D, _PD]),
    ("adv_ic_heat2d_gauss_noise", _I, [_I, _I, C.c_uint32, _D, _PD]),
    ("adv_ic_heat3d_blobs", _I, [_I, _I, _I, C.c_uint32, _I, _PD]),
    ("adv_ic_burgers_fourier", _I, [_I, _I, _I, _D, C.c_uint32, _I, _D, _PD]),
    ("adv_ic_burgers_ref", _I, [_I, _I, _I, _D, _D, _D, _PD]),
    ("adv_ic_burgers_ref2d", _I, [_I, _I, _D, _D, _PD]),
    ("adv_write_result_bin", _I, [C.c_char_p, _I, _VP, _I64]),
    ("adv_read_result_bin", _I, [C.c_char_p, _I64, _PD]),
    ("adv_strip_ghost_slabs", _I, [_I, _I, _I, _I, _PD, _PD]),
    ("adv_pad_ghost_slabs", _I, [_I, _I, _I, _I, _I, _PD, _PD]),
    ("adv_checkpoint_save", _I, [C.c_char_p, _I, _I, _I, _I, _I64, _D, _VP]),
    ("adv_checkpoint_load", _I, [C.c_char_p, C.POINTER(CheckpointHeader), _VP, C.c_size_t]),
    ("adv_crc32", C.c_uint32, [_VP, C.c_size_t]),
    ("adv_last_error_string", C.c_char_p, []),
    ("adv_status_string", C.c_char_p, [_I]),
    ("adv_abi_version", _I, []),
    ("adv_kernel_launch_count", C.c_int64, []),
    ("adv_ref_laplace", _I, [_I, _I, _I, _I, _I, _I64, _I, _I, _I, _D, _D, _D, _VP, _VP, _VP]),
    ("adv_ref_rk", _I, [_I, _I, _I, _I64, _I, _I, _I, _I, _D, _VP, _VP, _VP, _VP]),
    ("adv_ref_burgers_sweep", _I, [_I, _I, _I, _I64, _I, _I, _I, _D, _VP, _VP, _VP]),
    ("adv_ref_burgers_viscous", _I, [_I, _I64, _I, _I, _I, _D, _D, _D, _I, _VP, _VP, _VP]),
    ("adv_ref_laplace_box", _I, [_I, _I, _I, _VP, _I, _I, _I64, _I, _I, _I, _D, _D, _D, _VP, _VP, _VP]),
    ("adv_ref_burgers_sweep_all", _I, [_I, _I, _I, _I64, _I, _I, _I, _D, _VP, _VP, _VP]),
]


class AdvError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: status {status} ({msg})")
        self.status = status


_lib = None


def lib_path(name: str | None = None) -> Path:
    """The native library: libadvdiff.so, or the build named by ADVDIFF_LIBRARY (e.g.
    libadvdiff_checked.so, the bounds-checked build the tests run against)."""
    return LIBDIR / (name or os.environ.get("ADVDIFF_LIBRARY", "libadvdiff.so"))


def load() -> C.CDLL:
    """Loads libadvdiff.so once; raises if it has not been built."""
    global _lib
    if _lib is None:
        p = lib_path()
        if not p.exists():
            raise RuntimeError(f"{p} is missing: build the CUDA library first "
                               "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = C.CDLL(str(p), mode=os.RTLD_GLOBAL if hasattr(os, "RTLD_GLOBAL") else 0)
        for name, res, args in SIGNATURES:
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def check(status: int, where: str) -> None:
    if status != ADV_OK:
        msg = load().adv_last_error_string()
        raise AdvError(status, where, msg.decode() if msg else "")


def stream_handle(stream) -> int | None:
    """cudaStream_t of a torch.cuda.Stream (or an int handle), None for the default stream."""
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream
