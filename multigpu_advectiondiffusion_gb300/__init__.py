"""GB300-native (sm_103a) explicit solvers of wme7/MultiGPU_AdvectionDiffusion's single-GPU path.

* heat equation, 2D/3D: O2 5/7-point or O4 9/13-point Laplacian with forward Euler or SSP-RK3,
  one fused launch per stage (reference: SingleGPU/Diffusion{2d,3d}_*/kernels.cu);
* 3D Burgers: WENO5-JS / WENO5-Z reconstruction with local or global Lax-Friedrichs splitting
  fused into the SSP-RK3 stage, the time loop resident in one CUDA graph
  (reference: SingleGPU/Burgers3d_WENO5*/kernels.cu).

The compute path is the CUDA library ``_lib/libadvdiff.so`` (C ABI: include/advdiff.h);
``solvers`` wraps it for torch tensors. Build with ``multigpu_advectiondiffusion_gb300.build``.
"""
from . import _native  # noqa: F401
from .solvers import (BurgersConfig, HeatConfig, burgers_run, burgers_stage, heat_run, heat_stage,  # noqa: F401
                      max_abs)

__all__ = ["HeatConfig", "BurgersConfig", "heat_stage", "heat_run", "burgers_stage", "burgers_run", "max_abs"]
