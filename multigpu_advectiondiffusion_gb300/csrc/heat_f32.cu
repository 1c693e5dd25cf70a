// heat_f32.cu -- float-state instantiations of the fused heat stage (see heat_stage.cuh).
#include "heat_stage.cuh"

namespace adv {

// Kernel for (order, ndim, TMA or cp.async loads, stage specialisation, rows per thread, warps
// per CTA, lanes per row). Four rows per thread with 4 warps exist for the 3D O2 stencil with TMA
// loads, in rows of 32 lanes (tile 128 x 16) or 16 lanes (tile 64 x 32).
void* heat_kernel_f32(int order, int ndim, bool tma, int stage_kind, int rows, int warps, int lanes) {
  if (rows == 4) {
    if (order != 2 || ndim != 3 || !tma || warps != 4) return nullptr;
#define R4(L)                                                                                  \
  switch (stage_kind) {                                                                        \
    case 1: return reinterpret_cast<void*>(&heat_stage_kernel<float, 2, 3, true, 1, 4, 4, L>); \
    case 2: return reinterpret_cast<void*>(&heat_stage_kernel<float, 2, 3, true, 2, 4, 4, L>); \
    case 3: return reinterpret_cast<void*>(&heat_stage_kernel<float, 2, 3, true, 3, 4, 4, L>); \
    default: return reinterpret_cast<void*>(&heat_stage_kernel<float, 2, 3, true, 0, 4, 4, L>); \
  }
    if (lanes == 16) { R4(16) }
    R4(32)
#undef R4
  }
  if (warps != 8 || lanes != 32) return nullptr;
#define HK(O, N, M, S) reinterpret_cast<void*>(&heat_stage_kernel<float, O, N, M, S>)
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

// The failure-path test's variant of the FP32 3D O2 stage-1 kernel with TMA loads (4 rows, 4 warps,
// rows of `lanes` lanes): it withholds one plane's copy and takes the wait limit from its
// parameters (HeatParams::withheld_plane, wait_limit_ns).
void* heat_test_hook_kernel_f32(int lanes) {
  return lanes == 16 ? reinterpret_cast<void*>(&heat_stage_kernel<float, 2, 3, true, 1, 4, 4, 16, false, true>)
                     : reinterpret_cast<void*>(&heat_stage_kernel<float, 2, 3, true, 1, 4, 4, 32, false, true>);
}

}  // namespace adv
