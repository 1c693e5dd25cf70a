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
#define K(Z, D, V) reinterpret_cast<void*>(&burgers_batch_kernel<double, Z, D, V>)
  if (d.div == ADV_DIV_FAST) {  // common-denominator form, one division per side
    if (z) return visc ? K(true, FastDiv, true) : K(true, FastDiv, false);
    return visc ? K(false, FastDiv, true) : K(false, FastDiv, false);
  }
  if (z) return visc ? K(true, double, true) : K(true, double, false);
  return visc ? K(false, double, true) : K(false, double, false);
#undef K
}

}  // namespace adv
