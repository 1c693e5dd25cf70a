// heat_f64.cu -- double-state instantiations of the fused heat stage (see heat_stage.cuh).
#include "heat_stage.cuh"

namespace adv {

// Kernel for (order, ndim, TMA or cp.async loads, stage specialisation, the reference's rounding
// or the fused multiply-add form).
template <bool CT>
static void* heat_kernel_f64_t(int order, int ndim, bool tma, int stage_kind) {
#define HK(O, N, M, S) reinterpret_cast<void*>(&heat_stage_kernel<double, O, N, M, S, 2, 8, 32, CT>)
#define HS(O, N, M)                                            \
  switch (stage_kind) {                                        \
    case 1: return HK(O, N, M, 1);                             \
    case 2: return HK(O, N, M, 2);                             \
    case 3: return HK(O, N, M, 3);                             \
    default: return HK(O, N, M, 0);                            \
  }
  if (order == 2 && ndim == 3) { if (tma) { HS(2, 3, true) } else { HS(2, 3, false) } }
  if (order == 4 && ndim == 3) { if (tma) { HS(4, 3, true) } else { HS(4, 3, false) } }
  if (order == 2 && ndim == 2) { if (tma) { HS(2, 2, true) } else { HS(2, 2, false) } }
  if (order == 4 && ndim == 2) { if (tma) { HS(4, 2, true) } else { HS(4, 2, false) } }
#undef HS
#undef HK
  return nullptr;
}

void* heat_kernel_f64(int order, int ndim, bool tma, int stage_kind, int rows, int warps, int lanes, bool contract) {
  if (rows != 2 || warps != 8 || lanes != 32) return nullptr;
  return contract ? heat_kernel_f64_t<true>(order, ndim, tma, stage_kind)
                  : heat_kernel_f64_t<false>(order, ndim, tma, stage_kind);
}

}  // namespace adv
