// heat2_f32.cu -- instantiation of the two-step FP32 3D O2 heat kernel (see heat_twostep.cuh).
#include "heat_twostep.cuh"

namespace adv {

void* heat_twostep_kernel_ptr() { return reinterpret_cast<void*>(&heat_twostep_kernel); }
size_t heat_twostep_smem() { return Heat2Tile::SMEM; }

}  // namespace adv
