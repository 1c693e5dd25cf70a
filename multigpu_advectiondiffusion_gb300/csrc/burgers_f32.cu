// burgers_f32.cu -- FP32-state instantiations of the fused Burgers stage.
#include "burgers_launch.cuh"

namespace adv {

template <>
void* burgers_kernel_for<float>(const adv_burgers_desc& d) {
  const bool z = d.weno == ADV_WENO5_Z;
  const bool d64 = d.div == ADV_DIV_F64;
  const bool visc = d.kx != 0.0 || d.ky != 0.0 || d.kz != 0.0;
#define K(Z, D, V) reinterpret_cast<void*>(&burgers_stage_kernel<float, Z, D, V>)
  if (z) {
    if (d64) return visc ? K(true, double, true) : K(true, double, false);
    return visc ? K(true, float, true) : K(true, float, false);
  }
  if (d64) return visc ? K(false, double, true) : K(false, double, false);
  return visc ? K(false, float, true) : K(false, float, false);
#undef K
}

adv_status burgers_launch_f32(const adv_burgers_desc& d, const BurgersLaunch& L, const BurgersStageArgs& a,
                              cudaStream_t s) {
  return burgers_launch_t<float>(d, L, a, s);
}

size_t burgers_smem_f32() { return BurgersSmem<float>::TOTAL; }

}  // namespace adv
