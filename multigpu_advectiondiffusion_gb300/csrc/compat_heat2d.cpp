// compat_heat2d.cpp -- the reference's 2D heat wrapper names over the reference-semantics
// operators (include/advdiff_compat_heat2d.h). ADV_COMPAT_PITCHED selects the pitched variant.
#include "../../include/advdiff_compat_heat2d.h"

#include "../../include/advdiff_ref_ops.h"
#include "compat_common.h"

namespace {
double g_k[2] = {0.0, 0.0};  // the reference's __constant__ d_kx, d_ky
}

extern "C" {

void CopyToConstantMemory(const double kx, const double ky) {
  g_k[0] = kx;
  g_k[1] = ky;
}

#ifndef ADV_COMPAT_PITCHED
void Call_Lu2d(dim3, dim3, cudaStream_t s, unsigned int nx, unsigned int ny, double* u, double* Lu) {
  const unsigned int pitch = nx;
#else
void Call_Lu2d(dim3, dim3, cudaStream_t s, unsigned int pitch, unsigned int nx, unsigned int ny, double* u, double* Lu) {
#endif
  adv_compat::note(adv_ref_laplace(ADV_F64, 2, 4, 3, 1, pitch, nx, ny, 1, g_k[0], g_k[1], 0.0, u, Lu, s), "Call_Lu2d");
}

#ifndef ADV_COMPAT_PITCHED
void Call_RK2d(dim3, dim3, cudaStream_t s, unsigned int step, unsigned int nx, unsigned int ny, double dt, double* u,
               double* uo, double* Lu) {
  const unsigned int pitch = nx;
#else
void Call_RK2d(dim3, dim3, cudaStream_t s, unsigned int step, unsigned int pitch, unsigned int nx, unsigned int ny,
               double dt, double* u, double* uo, double* Lu) {
#endif
  adv_compat::note(adv_ref_rk(ADV_F64, 2, 3, pitch, nx, ny, 1, (int)step, dt, u, uo, Lu, s), "Call_RK2d");
}

int adv_compat_last_status(void) { return adv_compat::take_status(); }

}  // extern "C"
