// burgers_f32.cu -- FP32-state instantiations of the fused Burgers stage.
#include "burgers_launch.cuh"

namespace adv {

template <>
void* burgers_kernel_for<float>(const adv_burgers_desc& d) {
  const bool z = d.weno == ADV_WENO5_Z;
  const bool visc = d.kx != 0.0 || d.ky != 0.0 || d.kz != 0.0;
#define K(Z, D, V) reinterpret_cast<void*>(&burgers_stage_kernel<float, Z, D, V>)
#define KD(Z, V)                                          \
  switch (d.div) {                                        \
    case ADV_DIV_F64: return K(Z, double, V);             \
    case ADV_DIV_FAST: return K(Z, FastDiv, V);           \
    default: return K(Z, float, V);                       \
  }
  if (z) {
    if (visc) { KD(true, true) } else { KD(true, false) }
  } else {
    if (visc) { KD(false, true) } else { KD(false, false) }
  }
#undef KD
#undef K
}

adv_status burgers_launch_f32(const adv_burgers_desc& d, const BurgersLaunch& L, const BurgersStageArgs& a,
                              cudaStream_t s) {
  return burgers_launch_t<float>(d, L, a, s);
}

size_t burgers_smem_f32() { return BurgersSmem<float>::TOTAL; }

}  // namespace adv
