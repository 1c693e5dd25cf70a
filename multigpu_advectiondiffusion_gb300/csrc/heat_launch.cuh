// heat_launch.cuh -- host-side construction of the fused heat stage's parameters, shared by the
// single-grid launcher (heat_kernels.cu) and the batched ensembles (ensemble.cu).
#pragma once
#include "adv_internal.h"
#include "heat_stage.cuh"

namespace adv {

template <class T>
HeatParams<T> heat_params(const adv_heat_desc& d, const HeatLaunch& L, int stage, const void* u_in, const void* u_n,
                          void* u_out) {
  HeatParams<T> p;
  p.uin = static_cast<const T*>(u_in);
  p.un = static_cast<const T*>(u_n);
  p.out = static_cast<T*>(u_out);
  p.nx = d.nx; p.ny = d.ny; p.nz = d.ndim == 3 ? d.nz : 1;
  p.frozen = d.frozen; p.zero_boundary = d.zero_boundary; p.stage = stage;
  p.tiles_x = L.tiles_x;
  p.tiles_y = L.tiles_y;
  p.vec_ok = (((uintptr_t)u_out % 16) == 0 && ((int64_t)d.nx * sizeof(T)) % 16 == 0) ? 1 : 0;
  p.kx = (T)d.kx; p.ky = (T)d.ky; p.kz = (T)d.kz; p.dt = (T)d.dt;
  p.status = device_status_ptr();
  p.withheld_plane = L.withheld_plane;
  p.wait_limit_ns = L.wait_limit_ns ? L.wait_limit_ns : kWaitLimitNs;
  return p;
}

}  // namespace adv
