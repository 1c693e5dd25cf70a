"""Device-side failure reporting on the GPU, without a fault.

Every wait of the fused heat stage for a shared-memory copy is bounded; when one runs out the
kernel records ADV_ERR_TIMEOUT in the per-device status word, lets the copies it already issued
land, and returns. adv_test_heat_stage_withheld launches a stage in which one plane's copy is
never issued (a barrier phase nothing completes) with a 1 ms limit, so that path runs for real.
The caller learns of it through adv_device_status, and the context stays usable: the next
stage is bit-exact against the oracle. The reference instead prints and exits the process on
any CUDA error (SingleGPU/Burgers3d_WENO5/main.cpp:13-24).
"""
import ctypes as C
import time

import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import HeatConfig, heat_stage

pytestmark = pytest.mark.gpu


def test_withheld_copy_times_out_reports_and_leaves_the_gpu_usable(cuda, native, oracle):
    import torch
    n = 64
    cfg = HeatConfig.dirichlet_o2(3, n)
    d = cfg.desc(N.ADV_F32)
    u0 = oracle.ic_heat3d_blobs(n, n, n, 2).astype(np.float32)
    a = torch.from_numpy(u0).to(cuda)
    out = torch.full_like(a, float("nan"))
    torch.cuda.synchronize()
    assert native.adv_device_status(None) == N.ADV_OK  # nothing pending before the test
    t0 = time.perf_counter()
    st = native.adv_test_heat_stage_withheld(C.byref(d), 1, a.data_ptr(), a.data_ptr(), out.data_ptr(), 20,
                                             1_000_000, None)
    assert st == N.ADV_OK, native.adv_last_error_string()  # the launch itself succeeds
    assert native.adv_device_status(None) == N.ADV_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 10.0
    assert native.adv_device_status(None) == N.ADV_OK  # read once, then cleared
    assert torch.isnan(out).any().item()  # the stalled CTAs left their planes unwritten
    # the context is intact: the same stage now runs to completion, bit for bit
    out2 = torch.full_like(a, float("nan"))
    heat_stage(cfg, 1, a, a, out2)
    np.testing.assert_array_equal(out2.cpu().numpy(), oracle.heat_stage(cfg, 1, u0, u0))
    assert native.adv_device_status(None) == N.ADV_OK


def test_timeout_is_reported_by_the_next_synchronous_call(cuda, native, oracle):
    """adv_max_abs synchronises and reads the status word, so an earlier asynchronous stage's
    timeout surfaces there too."""
    import torch
    n = 48
    cfg = HeatConfig.dirichlet_o2(3, n)
    d = cfg.desc(N.ADV_F32)
    a = torch.from_numpy(oracle.ic_heat3d_blobs(n, n, n, 2).astype(np.float32)).to(cuda)
    out = torch.zeros_like(a)
    assert native.adv_test_heat_stage_withheld(C.byref(d), 1, a.data_ptr(), a.data_ptr(), out.data_ptr(), 0,
                                               200_000, None) == N.ADV_OK
    m = C.c_double(0.0)
    assert native.adv_max_abs(N.ADV_F32, a.data_ptr(), a.numel(), C.byref(m), None) == N.ADV_ERR_TIMEOUT
    assert native.adv_device_status(None) == N.ADV_OK
    assert native.adv_max_abs(N.ADV_F32, a.data_ptr(), a.numel(), C.byref(m), None) == N.ADV_OK
    assert m.value == float(a.abs().max())


def test_device_status_refuses_a_capturing_stream(cuda, native):
    import torch
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        g.capture_begin()
        try:
            assert native.adv_device_status(s.cuda_stream) == N.ADV_ERR_UNSUPPORTED
        finally:
            g.capture_end()
    assert native.adv_device_status(None) == N.ADV_OK
