"""Host-side argument checks of the Python solver surface (no GPU): every grid-shaped tensor
handed to the C ABI must be a contiguous CUDA tensor of the call's dtype and device with at
least the grid's element count, and caller-supplied work buffers must be large enough. The
checks run before any native call, so stand-in tensor objects exercise them on the CPU."""
from __future__ import annotations

import pytest
import torch

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300 import solvers as S


class FakeCuda:
    """Just enough of a CUDA tensor for the checks; its pointer is never dereferenced."""

    def __init__(self, n, dtype=torch.float32, device="cuda:0", contiguous=True):
        self._n, self.dtype, self.device, self._contig = n, dtype, torch.device(device), contiguous
        self.is_cuda = True

    def numel(self):
        return self._n

    def element_size(self):
        return torch.empty(0, dtype=self.dtype).element_size()

    def is_contiguous(self):
        return self._contig

    def data_ptr(self):
        return 0x10000


HEAT = S.HeatConfig.dirichlet_o2(3, 16)          # 4096 nodes
BURG = S.BurgersConfig.periodic(12)              # 1728 cells


def test_heat_stage_rejects_short_mixed_or_strided_fields():
    n = HEAT.numel
    with pytest.raises(ValueError, match="elements"):
        S.heat_stage(HEAT, 1, FakeCuda(n), FakeCuda(n), FakeCuda(n - 1))
    with pytest.raises(ValueError, match="dtype"):
        S.heat_stage(HEAT, 1, FakeCuda(n), FakeCuda(n), FakeCuda(n, torch.float64))
    with pytest.raises(ValueError, match="device"):
        S.heat_stage(HEAT, 1, FakeCuda(n), FakeCuda(n, device="cuda:1"), FakeCuda(n))
    with pytest.raises(ValueError, match="contiguous"):
        S.heat_stage(HEAT, 1, FakeCuda(n), FakeCuda(n, contiguous=False), FakeCuda(n))
    with pytest.raises(ValueError, match="CUDA"):
        S.heat_stage(HEAT, 1, torch.zeros(n), torch.zeros(n), torch.zeros(n))
    with pytest.raises(ValueError, match="unsupported dtype"):
        S.heat_stage(HEAT, 1, FakeCuda(n, torch.float16), FakeCuda(n, torch.float16), FakeCuda(n, torch.float16))


def test_heat_run_rejects_a_small_workspace():
    need = S._heat_workspace_bytes(HEAT, N.ADV_F32)
    assert need >= HEAT.numel * 4
    with pytest.raises(ValueError, match="bytes"):
        S.heat_run(HEAT, FakeCuda(HEAT.numel), 10, workspace=FakeCuda(need - 1, torch.uint8))
    with pytest.raises(ValueError, match="elements"):
        S.heat_run(HEAT, FakeCuda(HEAT.numel // 2), 10, workspace=FakeCuda(need, torch.uint8))


def test_burgers_calls_check_fields_key_and_workspace():
    n = BURG.numel
    with pytest.raises(ValueError, match="elements"):
        S.burgers_stage(BURG, 1, FakeCuda(n), FakeCuda(n - 5), FakeCuda(n), 1e-3)
    with pytest.raises(ValueError, match="int64"):
        S.burgers_stage(BURG, 1, FakeCuda(n, torch.float64), FakeCuda(n, torch.float64), FakeCuda(n, torch.float64),
                        1e-3, maxabs_key=FakeCuda(2, torch.int32))
    need = S._burgers_workspace_bytes(BURG, N.ADV_F64)
    with pytest.raises(ValueError, match="bytes"):
        S.burgers_run(BURG, FakeCuda(n, torch.float64), 0.1, 0.4, workspace=FakeCuda(need // 2, torch.uint8))
    one = (n * 4 + 255) // 256 * 256
    with pytest.raises(ValueError, match="bytes"):
        S.burgers_adjoint_step(BURG, FakeCuda(n), FakeCuda(n), FakeCuda(n), 1e-3, FakeCuda(n),
                               work=FakeCuda(3 * one - 1, torch.uint8))
    with pytest.raises(ValueError, match="dtype"):
        S.burgers_adjoint_step(BURG, FakeCuda(n), FakeCuda(n), FakeCuda(n), 1e-3, FakeCuda(n, torch.float64))


def test_heatk_and_ensemble_members_are_checked():
    cfg = S.HeatKConfig.cube(10, 0.1, 1.0)
    n = cfg.numel
    with pytest.raises(ValueError, match="elements"):
        S.heatk_step(cfg, FakeCuda(n - 1), FakeCuda(n), FakeCuda(n))
    with pytest.raises(ValueError, match="dtype"):
        S.heatk_adjoint_step(cfg, FakeCuda(n), FakeCuda(n), FakeCuda(n), FakeCuda(n), FakeCuda(n, torch.float64))
    with pytest.raises(ValueError, match="elements"):
        S.Ensemble(heat=[(HEAT, FakeCuda(HEAT.numel - 1))])
    with pytest.raises(ValueError, match="elements"):
        S.Ensemble(burgers=[(BURG, FakeCuda(10), 0.1, 0.4)])
    with pytest.raises(ValueError, match="at least one member"):
        S.Ensemble()


class FakeLib:
    """Records native calls and reports success (no GPU work is done)."""

    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def fn(*args):
            self.calls.append((name, args))
            return N.ADV_OK
        return fn


def test_valid_calls_reach_the_native_library(monkeypatch):
    """Every checked wrapper, given valid stand-in tensors, passes its pointers to the library."""
    fake = FakeLib()
    monkeypatch.setattr(N, "load", lambda: fake)
    n, nb = HEAT.numel, BURG.numel
    ws = FakeCuda(1 << 30, torch.uint8)
    S.heat_stage(HEAT, 1, FakeCuda(n), FakeCuda(n), FakeCuda(n))
    S.heat_run(HEAT, FakeCuda(n), 5, workspace=ws)
    d64 = torch.float64
    S.burgers_stage(BURG, 2, FakeCuda(nb, d64), FakeCuda(nb, d64), FakeCuda(nb, d64), 1e-3, 0.5,
                    maxabs_key=FakeCuda(1, torch.int64))
    S.burgers_run(BURG, FakeCuda(nb), 0.1, 0.4, workspace=ws)
    S.burgers_adjoint_step(BURG, FakeCuda(nb), FakeCuda(nb), FakeCuda(nb), 1e-3, FakeCuda(nb), work=ws)
    kc = S.HeatKConfig.cube(10, 0.1, 1.0)
    f = [FakeCuda(kc.numel) for _ in range(5)]
    S.heatk_step(kc, f[0], f[1], f[2])
    S.heatk_adjoint_step(kc, *f)
    S.autotune_heat(HEAT, FakeCuda(n))
    S.autotune_burgers(BURG, FakeCuda(nb))
    S.autotune_heatk(kc, f[0], f[1])
    S.max_abs(FakeCuda(n))
    names = [c[0] for c in fake.calls]
    for want in ("adv_heat_stage", "adv_heat_workspace_bytes", "adv_heat_run", "adv_burgers_stage",
                 "adv_burgers_workspace_bytes", "adv_burgers_run", "adv_burgers_adjoint_step", "adv_heatk_step",
                 "adv_heatk_adjoint_step", "adv_autotune_heat", "adv_autotune_burgers", "adv_autotune_heatk",
                 "adv_max_abs"):
        assert want in names, want
    stage = dict(fake.calls)["adv_burgers_stage"]
    assert stage[2:5] == (0x10000, 0x10000, 0x10000) and stage[7] == 0x10000  # fields and the key


def test_checkpoint_interval_keeps_the_run_when_it_fits():
    """The differentiable runs keep every state (interval = nsteps: no recompute in the backward
    run) when the kept arrays fit in half the free memory, else space checkpoints sqrt(N) apart."""
    one = 8 << 20                                  # one 128^3 FP32 array
    assert S.checkpoint_interval(400, 3, one, 1200 * one * 2) == 400      # exactly half the free memory
    assert S.checkpoint_interval(400, 3, one, 1200 * one * 2 - 1) == 20   # one byte short: sqrt(400)
    assert S.checkpoint_interval(200, 1, one, 10 * one) == S.default_interval(200) == 15
    assert S.checkpoint_interval(0, 1, one, 1 << 40) == 1
    assert S.default_interval(1) == 1 and S.default_interval(10) == 4
