// burgers_batch_f32.cu -- FP32-state instantiations of the batched Burgers stage
// (burgers_batch_kernel in burgers_kernels.cuh) used by the ensembles.
#include "burgers_kernels.cuh"
#include "adv_internal.h"

namespace adv {

template <class T>
void* burgers_batch_kernel_for(const adv_burgers_desc& d);

template <>
void* burgers_batch_kernel_for<float>(const adv_burgers_desc& d) {
  const bool z = d.weno == ADV_WENO5_Z;
  const bool visc = d.kx != 0.0 || d.ky != 0.0 || d.kz != 0.0;
#define K(Z, D, V) reinterpret_cast<void*>(&burgers_batch_kernel<float, Z, D, V>)
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

}  // namespace adv
