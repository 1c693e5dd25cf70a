// heat_batch.cu -- instantiations of the batched 3D heat stage (heat_batch_kernel in
// heat_stage.cuh) used by the ensembles.
#include "adv_internal.h"
#include "heat_stage.cuh"

namespace adv {

// Kernel for (state type, order, TMA or cp.async loads, stage specialisation 1..3, rows per
// thread, lanes per row). Four rows per thread (4 warps; rows of 32 or 16 lanes) exist for FP32
// O2 with TMA loads.
void* heat_batch_kernel_for(int dtype, int order, bool tma, int stage_kind, int rows, int lanes) {
  if (rows == 4) {
    if (dtype != ADV_F32 || order != 2 || !tma) return nullptr;
#define B4(L)                                                                                 \
  switch (stage_kind) {                                                                       \
    case 1: return reinterpret_cast<void*>(&heat_batch_kernel<float, 2, true, 1, 4, 4, L>);   \
    case 2: return reinterpret_cast<void*>(&heat_batch_kernel<float, 2, true, 2, 4, 4, L>);   \
    case 3: return reinterpret_cast<void*>(&heat_batch_kernel<float, 2, true, 3, 4, 4, L>);   \
    default: return nullptr;                                                                  \
  }
    if (lanes == 16) { B4(16) }
    B4(32)
#undef B4
  }
  if (lanes != 32) return nullptr;
#define HB(T, O, M, S) reinterpret_cast<void*>(&heat_batch_kernel<T, O, M, S>)
#define HS(T, O, M)                  \
  switch (stage_kind) {              \
    case 1: return HB(T, O, M, 1);   \
    case 2: return HB(T, O, M, 2);   \
    case 3: return HB(T, O, M, 3);   \
    default: return nullptr;         \
  }
#define HM(T, O) if (tma) { HS(T, O, true) } else { HS(T, O, false) }
  if (dtype == ADV_F32) {
    if (order == 2) { HM(float, 2) }
    if (order == 4) { HM(float, 4) }
  } else if (dtype == ADV_F64) {
    if (order == 2) { HM(double, 2) }
    if (order == 4) { HM(double, 4) }
  }
#undef HM
#undef HS
#undef HB
  return nullptr;
}

// The two-width kernel (4-row FP32 O2 tiles of 128 and 64 nodes, TMA loads) for stage 1..3.
void* heat_batch_mixed_kernel_for(int stage_kind) {
  switch (stage_kind) {
    case 1: return reinterpret_cast<void*>(&heat_batch_mixed_kernel<1>);
    case 2: return reinterpret_cast<void*>(&heat_batch_mixed_kernel<2>);
    case 3: return reinterpret_cast<void*>(&heat_batch_mixed_kernel<3>);
    default: return nullptr;
  }
}

size_t heat_batch_inst_bytes(int dtype) {
  return dtype == ADV_F32 ? sizeof(HeatBatchInst<float>) : sizeof(HeatBatchInst<double>);
}

}  // namespace adv
