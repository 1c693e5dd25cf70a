// burgers_f64.cu -- FP64-state instantiations of the fused Burgers stage (the reference's own
// precision): reconstruction in the reference's operand order, bit-exact against the oracle,
// or, with ADV_DIV_FAST, the common-denominator form (one division per WENO side).
#include "burgers_launch.cuh"

namespace adv {

template <>
void* burgers_kernel_for<double>(const adv_burgers_desc& d) {
  const bool z = d.weno == ADV_WENO5_Z;
  const bool visc = d.kx != 0.0 || d.ky != 0.0 || d.kz != 0.0;
#define K(Z, D, V) reinterpret_cast<void*>(&burgers_stage_kernel<double, Z, D, V>)
  if (d.div == ADV_DIV_FAST) {  // common-denominator form, one division per side
    if (z) return visc ? K(true, FastDiv, true) : K(true, FastDiv, false);
    return visc ? K(false, FastDiv, true) : K(false, FastDiv, false);
  }
  if (z) return visc ? K(true, double, true) : K(true, double, false);
  return visc ? K(false, double, true) : K(false, double, false);
#undef K
}

adv_status burgers_launch_f64(const adv_burgers_desc& d, const BurgersLaunch& L, const BurgersStageArgs& a,
                              cudaStream_t s) {
  return burgers_launch_t<double>(d, L, a, s);
}

size_t burgers_smem_f64() { return BurgersSmem<double>::TOTAL; }

}  // namespace adv
