"""adv_heat_run_noalloc through the C ABI, against adv_heat_run.

This entry point serves callers that cannot allocate device memory -- hosts whose device memory
belongs to their own allocator, and loops that must not call cudaMalloc/cudaFree because those
calls may synchronise the device. It keeps its intermediate state in one fixed device array
instead of a workspace, so it must give exactly the results of adv_heat_run (heat results are
bit-exact everywhere in these tests), call after call, without allocating. The file sorts last
so that a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import HeatConfig

pytestmark = pytest.mark.gpu


def _cases():
    return [
        ("3d-o2-euler-f32", HeatConfig.dirichlet_o2(3, 64), np.float32, 37),
        ("3d-o4-rk3-f64", HeatConfig.reference_3d(1.0, 10, 10, 10, 41, 39, 37), np.float64, 5),
        ("2d-o4-rk3-f64", HeatConfig.reference_2d(1.0, 10, 10, 301, 257), np.float64, 9),
        ("2d-o2-euler-f32-odd-rows", HeatConfig.dirichlet_o2(2, 333), np.float32, 40),
    ]


def _initial(cfg, dtype):
    rng = np.random.default_rng(cfg.nx * 7 + cfg.ny)
    u = rng.random(cfg.numel)
    return u.astype(dtype)


@pytest.mark.parametrize("name,cfg,dtype,nsteps", _cases(), ids=[c[0] for c in _cases()])
def test_noalloc_matches_heat_run_on_consecutive_calls(cuda, native, name, cfg, dtype, nsteps):
    import torch
    d = cfg.desc(N.ADV_F32 if dtype == np.float32 else N.ADV_F64)
    nb = C.c_size_t(0)
    assert native.adv_heat_workspace_bytes(C.byref(d), cfg.time, C.byref(nb)) == N.ADV_OK
    assert nb.value <= (16 << 20)
    ws = torch.empty(nb.value, dtype=torch.uint8, device=cuda)
    u0 = torch.from_numpy(_initial(cfg, dtype)).to(cuda)
    a = torch.empty_like(u0)
    b = torch.empty_like(u0)
    torch.cuda.synchronize()
    pool = _default_pool_reserved(cuda)
    for call in range(2):
        a.copy_(u0)
        b.copy_(u0)
        assert native.adv_heat_run(C.byref(d), cfg.time, nsteps, a.data_ptr(), ws.data_ptr(), None) == N.ADV_OK
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(cuda)[0]
        st = native.adv_heat_run_noalloc(C.byref(d), cfg.time, nsteps, b.data_ptr(), None)
        assert st == N.ADV_OK, native.adv_last_error_string()
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(cuda)[0]
        assert torch.equal(a, b), f"call {call}: results differ from adv_heat_run"
        if call == 1:  # set-up done on the first call: the second one takes no device memory
            assert free_after >= free_before
    # nothing came from the stream-ordered allocator's default pool either (cudaMallocAsync); the
    # pool may only have shrunk (memory an earlier test freed is released at synchronisation)
    after = _default_pool_reserved(cuda)
    assert pool is None or after <= pool


def _default_pool_reserved(dev):
    """Reserved bytes of the device's default memory pool (cudaMallocAsync), read through the
    CUDA runtime the library itself links; None if that runtime cannot be opened."""
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = C.CDLL(name)
            break
        except OSError:
            rt = None
    if rt is None:
        return None
    pool = C.c_void_p()
    if rt.cudaDeviceGetDefaultMemPool(C.byref(pool), C.c_int(dev.index or 0)) != 0:
        return None
    val = C.c_uint64(0)
    cudaMemPoolAttrReservedMemCurrent = 5
    if rt.cudaMemPoolGetAttribute(pool, C.c_int(cudaMemPoolAttrReservedMemCurrent), C.byref(val)) != 0:
        return None
    return val.value


def test_noalloc_rejects_runs_beyond_its_scratch(cuda, native):
    cfg = HeatConfig.dirichlet_o2(3, 256)  # 64 MiB of FP32 state > 16 MiB of scratch
    d = cfg.desc(N.ADV_F32)
    import torch
    u = torch.zeros(cfg.numel, device=cuda)
    st = native.adv_heat_run_noalloc(C.byref(d), cfg.time, 3, u.data_ptr(), None)
    assert st == N.ADV_ERR_INVALID_ARG
    msg = native.adv_last_error_string().decode()
    assert "scratch" in msg and str(16 << 20) in msg
    assert torch.count_nonzero(u).item() == 0
