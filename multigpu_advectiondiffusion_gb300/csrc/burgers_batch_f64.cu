// burgers_batch_f64.cu -- FP64-state instantiations of the batched Burgers stage
// (burgers_batch_kernel in burgers_kernels.cuh) used by the ensembles.
#include "burgers_kernels.cuh"
#include "adv_internal.h"

namespace adv {

template <class T>
void* burgers_batch_kernel_for(const adv_burgers_desc& d);

template <>
void* burgers_batch_kernel_for<double>(const adv_burgers_desc& d) {
  const bool z = d.weno == ADV_WENO5_Z;
  const bool visc = d.kx != 0.0 || d.ky != 0.0 || d.kz != 0.0;
#define K(Z, V) reinterpret_cast<void*>(&burgers_batch_kernel<double, Z, double, V>)
  if (z) return visc ? K(true, true) : K(true, false);
  return visc ? K(false, true) : K(false, false);
#undef K
}

}  // namespace adv
