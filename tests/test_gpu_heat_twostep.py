"""The two-step heat kernel (two forward-Euler steps per pass over HBM, FP32 3D O2) against the
oracle, bit for bit.

adv_heat_run takes this path for every FP32 3D O2 forward-Euler run whose rows are whole 16-byte
vectors; each launch must equal two single fused stages exactly (same fused multiply-add pattern),
so the whole run equals the oracle's step-by-step loop. Cases cover ragged tiles in x, y and z,
grids smaller than one tile, one and two frozen layers with and without the Dirichlet zero, random
data (every node's value matters), and every remainder of the step count modulo 4 (two-step
launches in pairs, then two-step and single-step launches for the rest).
"""
import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import HeatConfig, heat_run

pytestmark = pytest.mark.gpu

SIZES = [(64, 40, 24), (36, 29, 23), (128, 16, 10), (132, 70, 9), (8, 7, 6), (192, 33, 40), (260, 18, 11),
         (256, 48, 13)]


def _cfg(nx, ny, nz, frozen, zero):
    rng = np.random.default_rng(nx * 131 + ny * 7 + nz)
    k = rng.uniform(0.01, 0.05, 3)
    return HeatConfig(3, nx, ny, nz, 2, frozen, zero, *k, 0.7, N.ADV_EULER)


@pytest.mark.parametrize("size", SIZES)
@pytest.mark.parametrize("frozen,zero", [(1, True), (2, False), (1, False)])
@pytest.mark.parametrize("nsteps", [2, 5, 8])
def test_two_step_runs_equal_the_oracle(cuda, oracle, size, frozen, zero, nsteps):
    import torch
    nx, ny, nz = size
    if min(size) < 2 * frozen + 1:
        pytest.skip("grid smaller than its frozen layers")
    cfg = _cfg(nx, ny, nz, frozen, zero)
    u0 = np.random.default_rng(nsteps).standard_normal(nx * ny * nz).astype(np.float32)
    want = oracle.heat_run(cfg, u0, nsteps, 0)
    u = torch.from_numpy(u0).to(cuda)
    heat_run(cfg, u, nsteps)
    np.testing.assert_array_equal(u.cpu().numpy(), want)


@pytest.mark.parametrize("nsteps", [1, 2, 3, 4, 6, 7, 9, 10, 11, 129, 130, 131, 132])
def test_every_step_count_remainder(cuda, oracle, nsteps):
    """Remainders 0..3 of the step count, inside and past one captured chunk of launches."""
    import torch
    cfg = HeatConfig.dirichlet_o2(3, 40)
    u0 = oracle.ic_heat3d_blobs(40, 40, 40, 2).astype(np.float32)
    want = oracle.heat_run(cfg, u0, nsteps, 0)
    u = torch.from_numpy(u0).to(cuda)
    heat_run(cfg, u, nsteps)
    np.testing.assert_array_equal(u.cpu().numpy(), want)


def test_two_step_run_at_the_benchmark_size(cuda, oracle):
    """256^3, the benchmark's problem: 12 steps (6 two-step launches) equal the oracle."""
    import torch
    n = 256
    cfg = HeatConfig.dirichlet_o2(3, n)
    u0 = oracle.ic_heat3d_blobs(n, n, n, 2).astype(np.float32)
    want = oracle.heat_run(cfg, u0, 12, 0)
    u = torch.from_numpy(u0).to(cuda)
    heat_run(cfg, u, 12)
    np.testing.assert_array_equal(u.cpu().numpy(), want)
