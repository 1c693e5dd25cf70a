"""2D forward-Euler runs (adv_heat_run), which in FP32 advance up to eight steps per launch by
overlapped temporal tiling in shared memory, against the oracle's step-by-step loop, bit for bit
(FP64, rounded as written and contracted, keeps one step per launch and is checked the same way):
O2 and O4, held and zeroed boundaries, one to three
frozen layers, grids smaller than one 32 x 32 tile and spanning several, and every remainder of
the step count modulo 8 (full launches in captured pairs, an odd full launch, a shorter last one).
"""
import numpy as np
import pytest

from multigpu_advectiondiffusion_gb300 import _native as N
from multigpu_advectiondiffusion_gb300.solvers import HeatConfig, heat_run

pytestmark = pytest.mark.gpu


def _cfg(order, nx, ny, frozen, zero, contract=False):
    rng = np.random.default_rng(nx * 7 + ny)
    k = rng.uniform(0.01, 0.05, 2)
    return HeatConfig(2, nx, ny, 1, order, frozen, zero, k[0], k[1], 0.0, 0.7, N.ADV_EULER, contract=contract)


@pytest.mark.parametrize("size", [(64, 40), (37, 29), (7, 6), (300, 17), (97, 130)])
@pytest.mark.parametrize("order,frozen,zero", [(2, 1, True), (2, 2, False), (4, 2, True), (4, 3, False)])
@pytest.mark.parametrize("dtype,contract", [(np.float32, False), (np.float64, False), (np.float64, True)],
                         ids=["f32", "f64", "f64-contract"])
@pytest.mark.parametrize("nsteps", [2, 9, 23])
def test_heat2d_runs_equal_the_oracle(cuda, oracle, size, order, frozen, zero, dtype, contract, nsteps):
    import torch
    nx, ny = size
    if min(size) < 2 * frozen + 1:
        pytest.skip("grid smaller than its frozen layers")
    cfg = _cfg(order, nx, ny, frozen, zero, contract)
    u0 = np.random.default_rng(nsteps).standard_normal(nx * ny).astype(dtype)
    want = oracle.heat_run(cfg, u0, nsteps, 0)
    u = torch.from_numpy(u0).to(cuda)
    heat_run(cfg, u, nsteps)
    np.testing.assert_array_equal(u.cpu().numpy(), want)


@pytest.mark.parametrize("nsteps", [1, 7, 8, 15, 16, 17, 24, 31, 513, 1000])
def test_every_launch_count_remainder_at_the_benchmark_size(cuda, oracle, nsteps):
    """512^2 (the 2D configuration), step counts around multiples of 8 and 16, and past one
    captured chunk of launches."""
    import torch
    cfg = HeatConfig.dirichlet_o2(2, 512)
    u0 = oracle.ic_heat2d_gauss_noise(512, 512, 1, 1e-3).astype(np.float32)
    want = oracle.heat_run(cfg, u0, nsteps, 0)
    u = torch.from_numpy(u0).to(cuda)
    heat_run(cfg, u, nsteps)
    np.testing.assert_array_equal(u.cpu().numpy(), want)
