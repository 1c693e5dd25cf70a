"""The two-step heat kernel (two forward-Euler steps per pass over HBM, FP32 3D O2) against the
oracle, bit for bit.

adv_heat_run takes this path for an FP32 3D O2 forward-Euler problem whose rows are whole 16-byte
vectors when the tuning table says two steps per launch were faster for it (adv_autotune_heat
measures that); here the table entry is imported directly, so the path runs whatever the
measurement on this GPU. Each launch must equal two single fused stages exactly (same fused
multiply-add pattern), so the whole run equals the oracle's step-by-step loop. Cases cover ragged
tiles in x, y and z, grids smaller than one tile, one and two frozen layers with and without the
Dirichlet zero, random data (every node's value matters), and every remainder of the step count
modulo 4 (two-step launches in pairs, then two-step and single-step launches for the rest).
"""
import ctypes as C
import json

import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import HeatConfig, heat_run

pytestmark = pytest.mark.gpu

TUNE_HEAT_STEPS = 5


def _two_steps_per_launch(native, cfg):
    """Imports the tuning-table entry that makes adv_heat_run launch two steps at a time for cfg."""
    variant = N.ADV_F32 * 100 + cfg.order * 10 + cfg.ndim
    table = {"advdiff_autotune": 1, "entries": [{"kind": TUNE_HEAT_STEPS, "variant": variant, "nx": cfg.nx,
                                                 "ny": cfg.ny, "nz": cfg.nz, "a": 2, "b": 1}]}
    assert native.adv_autotune_import(json.dumps(table).encode()) == N.ADV_OK


@pytest.fixture(autouse=True)
def _clean_table(native):
    yield
    assert native.adv_autotune_clear() == N.ADV_OK

SIZES = [(64, 40, 24), (36, 29, 23), (128, 16, 10), (132, 70, 9), (8, 7, 6), (192, 33, 40), (260, 18, 11),
         (256, 48, 13)]


def _cfg(nx, ny, nz, frozen, zero):
    rng = np.random.default_rng(nx * 131 + ny * 7 + nz)
    k = rng.uniform(0.01, 0.05, 3)
    return HeatConfig(3, nx, ny, nz, 2, frozen, zero, *k, 0.7, N.ADV_EULER)


@pytest.mark.parametrize("size", SIZES)
@pytest.mark.parametrize("frozen,zero", [(1, True), (2, False), (1, False)])
@pytest.mark.parametrize("nsteps", [2, 5, 8])
def test_two_step_runs_equal_the_oracle(cuda, native, oracle, size, frozen, zero, nsteps):
    import torch
    nx, ny, nz = size
    if min(size) < 2 * frozen + 1:
        pytest.skip("grid smaller than its frozen layers")
    cfg = _cfg(nx, ny, nz, frozen, zero)
    u0 = np.random.default_rng(nsteps).standard_normal(nx * ny * nz).astype(np.float32)
    want = oracle.heat_run(cfg, u0, nsteps, 0)
    _two_steps_per_launch(native, cfg)
    u = torch.from_numpy(u0).to(cuda)
    heat_run(cfg, u, nsteps)
    np.testing.assert_array_equal(u.cpu().numpy(), want)


@pytest.mark.parametrize("nsteps", [1, 2, 3, 4, 6, 7, 9, 10, 11, 129, 130, 131, 132])
def test_every_step_count_remainder(cuda, native, oracle, nsteps):
    """Remainders 0..3 of the step count, inside and past one captured chunk of launches."""
    import torch
    cfg = HeatConfig.dirichlet_o2(3, 40)
    u0 = oracle.ic_heat3d_blobs(40, 40, 40, 2).astype(np.float32)
    want = oracle.heat_run(cfg, u0, nsteps, 0)
    _two_steps_per_launch(native, cfg)
    u = torch.from_numpy(u0).to(cuda)
    heat_run(cfg, u, nsteps)
    np.testing.assert_array_equal(u.cpu().numpy(), want)


def test_two_step_run_at_the_benchmark_size(cuda, native, oracle):
    """256^3, the benchmark's problem: 12 steps (6 two-step launches) equal the oracle."""
    import torch
    n = 256
    cfg = HeatConfig.dirichlet_o2(3, n)
    u0 = oracle.ic_heat3d_blobs(n, n, n, 2).astype(np.float32)
    want = oracle.heat_run(cfg, u0, 12, 0)
    _two_steps_per_launch(native, cfg)
    u = torch.from_numpy(u0).to(cuda)
    heat_run(cfg, u, 12)
    np.testing.assert_array_equal(u.cpu().numpy(), want)


def test_tuner_decides_the_steps_per_launch(cuda, native, oracle):
    """adv_autotune_heat records, for a two-step-eligible problem, how many steps a launch advances
    (1 or 2: whichever it measured faster), and a run after it equals the oracle either way."""
    import torch
    from multigpu_advectiondiffusion_gb300.solvers import autotune_heat
    n = 96
    cfg = HeatConfig.dirichlet_o2(3, n)
    u0 = oracle.ic_heat3d_blobs(n, n, n, 2).astype(np.float32)
    u = torch.from_numpy(u0).to(cuda)
    autotune_heat(cfg, u)
    size = C.c_size_t(0)
    assert native.adv_autotune_export(None, 0, C.byref(size)) == N.ADV_OK
    buf = C.create_string_buffer(size.value)
    assert native.adv_autotune_export(buf, size.value, C.byref(size)) == N.ADV_OK
    entries = [e for e in json.loads(buf.value.decode())["entries"] if e["kind"] == TUNE_HEAT_STEPS]
    assert len(entries) == 1 and entries[0]["a"] in (1, 2) and (entries[0]["nx"], entries[0]["nz"]) == (n, n)
    heat_run(cfg, u, 10)
    np.testing.assert_array_equal(u.cpu().numpy(), oracle.heat_run(cfg, u0, 10, 0))
