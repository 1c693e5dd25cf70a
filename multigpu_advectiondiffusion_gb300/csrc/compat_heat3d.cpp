// compat_heat3d.cpp -- the reference's 3D heat wrapper names over the reference-semantics
// operators (include/advdiff_compat_heat3d.h). ADV_COMPAT_PITCHED selects the pitched variant.
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

#ifndef ADV_COMPAT_PITCHED
void Call_Lu3d(dim3, dim3, cudaStream_t s, unsigned int nx, unsigned int ny, unsigned int nz, double* u, double* Lu) {
  const unsigned int pitch = nx;
#else
void Call_Lu3d(dim3, dim3, cudaStream_t s, unsigned int pitch, unsigned int nx, unsigned int ny, unsigned int nz,
               double* u, double* Lu) {
#endif
  adv_compat::note(adv_ref_laplace(ADV_F64, 3, 4, 2, 0, pitch, nx, ny, nz, g_k[0], g_k[1], g_k[2], u, Lu, s), "Call_Lu3d");
}

#ifndef ADV_COMPAT_PITCHED
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
