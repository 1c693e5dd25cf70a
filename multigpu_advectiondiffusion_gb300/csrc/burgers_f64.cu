// burgers_f64.cu -- FP64-state instantiations of the fused Burgers stage (the reference's own
// precision; reconstruction in the reference's operand order, bit-exact against the oracle).
#include "burgers_launch.cuh"

namespace adv {

template <>
void* burgers_kernel_for<double>(const adv_burgers_desc& d) {
  const bool z = d.weno == ADV_WENO5_Z;
  const bool visc = d.kx != 0.0 || d.ky != 0.0 || d.kz != 0.0;
#define K(Z, V) reinterpret_cast<void*>(&burgers_stage_kernel<double, Z, double, V>)
  if (z) return visc ? K(true, true) : K(true, false);
  return visc ? K(false, true) : K(false, false);
#undef K
}

adv_status burgers_launch_f64(const adv_burgers_desc& d, const BurgersLaunch& L, const BurgersStageArgs& a,
                              cudaStream_t s) {
  return burgers_launch_t<double>(d, L, a, s);
}

size_t burgers_smem_f64() { return BurgersSmem<double>::TOTAL; }

}  // namespace adv
