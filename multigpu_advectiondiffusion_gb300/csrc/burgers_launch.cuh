// burgers_launch.cuh -- host-side launch of the fused Burgers stage for one state type.
// Included by burgers_f32.cu and burgers_f64.cu so the two precisions compile in parallel.
#pragma once
#include "adv_internal.h"
#include "burgers_kernels.cuh"

namespace adv {

template <class T>
void* burgers_kernel_for(const adv_burgers_desc& d);

// Stage parameters of one launch (or of one instance of a batched launch).
template <class T>
BurgersParams<T> burgers_params(const adv_burgers_desc& d, const BurgersLaunch& L, const BurgersStageArgs& a) {
  BurgersParams<T> p;
  p.uin = static_cast<const T*>(a.u_in);
  p.un = static_cast<const T*>(a.u_n);
  p.out = static_cast<T*>(a.u_out);
  p.nx = d.nx; p.ny = d.ny; p.nz = d.nz;
  p.stage = a.stage;
  p.periodic = d.bc == ADV_BC_PERIODIC ? 1 : 0;
  p.bug_b2 = d.bug_b2;
  p.tiles_x = L.tiles_x;
  p.tiles_y = L.tiles_y;
  p.tma = L.tma ? 1 : 0;
  p.un_is_uin = a.u_n == a.u_in ? 1 : 0;
  p.lf_global = d.lf == ADV_LF_GLOBAL ? 1 : 0;
  p.dx = d.dx; p.dy = d.dy; p.dz = d.dz;
  p.kx = (T)d.kx; p.ky = (T)d.ky; p.kz = (T)d.kz;
  p.dt_host = a.dt_host;
  p.alpha_host = a.alpha_host;
  p.dt_dev = a.dt_dev;
  p.alpha_dev = a.alpha_dev;
  p.alpha_key = a.alpha_key;
  p.maxabs_key = a.maxabs_key;
  p.active = a.active;
  p.status = device_status_ptr();
  return p;
}

template <class T>
adv_status burgers_launch_t(const adv_burgers_desc& d, const BurgersLaunch& L, const BurgersStageArgs& a,
                            cudaStream_t s) {
  BurgersParams<T> p = burgers_params<T>(d, L, a);
  void* k = burgers_kernel_for<T>(d);
  if (!k) return set_error(ADV_ERR_UNSUPPORTED, "burgers: no kernel for this configuration");
  void* args[] = {const_cast<CUtensorMap*>(&L.tmap_in), &p};
  ADV_CUDA_TRY(cudaLaunchKernel(k, L.grid, L.block, args, L.smem, s));
  count_launches(1);
  return ADV_OK;
}

}  // namespace adv
