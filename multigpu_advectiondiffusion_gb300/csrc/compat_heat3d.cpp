// compat_heat3d.cpp -- the reference's 3D heat wrapper names over the reference-semantics
// operators (include/advdiff_compat_heat3d.h). ADV_COMPAT_PITCHED selects the pitched variant,
// ADV_COMPAT_BLOCKING the z-blocked one (pitched signatures, its own Laplacian node range).
#include "../../include/advdiff_compat_heat3d.h"

#include "../../include/advdiff_ref_ops.h"
#include "compat_common.h"

namespace {
double g_k[3] = {0.0, 0.0, 0.0};  // the reference's __constant__ d_kx, d_ky, d_kz
}

extern "C" {

void CopyToConstantMemory(double kx, double ky, double kz) {
  g_k[0] = kx;
  g_k[1] = ky;
  g_k[2] = kz;
}

#if defined(ADV_COMPAT_BLOCKING)
// SingleGPU/Diffusion3d_Blocking/kernels.cu:37-88, 167-171: 16-plane z blocks from kstart 3 to
// kstop nz-2, i and j in [3, n-4], operands west/south/bottom first. (Its first plane of a block is written without the kstop test;
// for the sizes where that plane is nz-2 or nz-1 the node is outside the RK range and the value
// is never read, so it is not reproduced.)
void Call_Lu3d(dim3, dim3, cudaStream_t s, unsigned int pitch, unsigned int nx, unsigned int ny, unsigned int nz,
               double* u, double* Lu) {
  const int32_t box[6] = {3, (int32_t)nx - 3, 3, (int32_t)ny - 3, 3, (int32_t)nz - 2};
  adv_compat::note(adv_ref_laplace_box(ADV_F64, 3, 4, box, 0, 1, pitch, nx, ny, nz, g_k[0], g_k[1], g_k[2], u, Lu, s),
                   "Call_Lu3d");
}
#else
#ifndef ADV_COMPAT_PITCHED
void Call_Lu3d(dim3, dim3, cudaStream_t s, unsigned int nx, unsigned int ny, unsigned int nz, double* u, double* Lu) {
  const unsigned int pitch = nx;
#else
void Call_Lu3d(dim3, dim3, cudaStream_t s, unsigned int pitch, unsigned int nx, unsigned int ny, unsigned int nz,
               double* u, double* Lu) {
#endif
  adv_compat::note(adv_ref_laplace(ADV_F64, 3, 4, 2, 0, pitch, nx, ny, nz, g_k[0], g_k[1], g_k[2], u, Lu, s), "Call_Lu3d");
}
#endif

#if !defined(ADV_COMPAT_PITCHED) && !defined(ADV_COMPAT_BLOCKING)
void Call_RK3d(dim3, dim3, cudaStream_t s, unsigned int step, unsigned int nx, unsigned int ny, unsigned int nz,
               double dt, double* u, double* uo, double* Lu) {
  const unsigned int pitch = nx;
#else
void Call_RK3d(dim3, dim3, cudaStream_t s, unsigned int step, unsigned int pitch, unsigned int nx, unsigned int ny,
               unsigned int nz, double dt, double* u, double* uo, double* Lu) {
#endif
  adv_compat::note(adv_ref_rk(ADV_F64, 3, 2, pitch, nx, ny, nz, (int)step, dt, u, uo, Lu, s), "Call_RK3d");
}

int adv_compat_last_status(void) { return adv_compat::take_status(); }

}  // extern "C"
