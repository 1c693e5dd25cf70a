// compat_burgers3d.cpp -- the reference's Burgers wrapper names over the reference-semantics
// operators (include/advdiff_compat_burgers3d.h). ADV_COMPAT_PITCHED selects the pitched variant;
// with ADV_COMPAT_SHAREDMEM as well, the shared-memory program's sweeps.
#include "../../include/advdiff_compat_burgers3d.h"

#include <atomic>

#include "../../include/advdiff_ref_ops.h"
#include "compat_common.h"

namespace {
double g_k[3] = {0.0, 0.0, 0.0};  // the reference's __constant__ d_kx, d_ky, d_kz
std::atomic<int> g_bug_b2{1};
}

#ifndef ADV_COMPAT_PITCHED
#define PITCH_PARAM
#define PITCH_VALUE Nx
#else
#define PITCH_PARAM unsigned int pitch,
#define PITCH_VALUE pitch
#endif

#ifdef ADV_COMPAT_SHAREDMEM
#define SWEEP adv_ref_burgers_sweep_all
#else
#define SWEEP adv_ref_burgers_sweep
#endif

extern "C" {

void CopyToConstantMemory(double kx, double ky, double kz) {
  g_k[0] = kx;
  g_k[1] = ky;
  g_k[2] = kz;
}

void Call_Adv_x(dim3, dim3, cudaStream_t s, PITCH_PARAM unsigned int Nx, unsigned int Ny, unsigned int Nz, double dx,
                double* u, double* Lu) {
  adv_compat::note(SWEEP(ADV_F64, 0, ADV_WENO5_Z, PITCH_VALUE, Nx, Ny, Nz, dx, u, Lu, s), "Call_Adv_x");
}
void Call_Adv_y(dim3, dim3, cudaStream_t s, PITCH_PARAM unsigned int Nx, unsigned int Ny, unsigned int Nz, double dy,
                double* v, double* Lv) {
  adv_compat::note(SWEEP(ADV_F64, 1, ADV_WENO5_Z, PITCH_VALUE, Nx, Ny, Nz, dy, v, Lv, s), "Call_Adv_y");
}
void Call_Adv_z(dim3, dim3, cudaStream_t s, PITCH_PARAM unsigned int Nx, unsigned int Ny, unsigned int Nz, double dz,
                double* w, double* Lw) {
  adv_compat::note(SWEEP(ADV_F64, 2, ADV_WENO5_Z, PITCH_VALUE, Nx, Ny, Nz, dz, w, Lw, s), "Call_Adv_z");
}
void Call_Diff_(dim3, dim3, cudaStream_t s, PITCH_PARAM unsigned int Nx, unsigned int Ny, unsigned int Nz, double* q,
                double* Lq) {
  adv_compat::note(adv_ref_burgers_viscous(ADV_F64, PITCH_VALUE, Nx, Ny, Nz, g_k[0], g_k[1], g_k[2], g_bug_b2.load(), q,
                                           Lq, s),
                   "Call_Diff_");
}
void Call_sspRK(dim3, dim3, cudaStream_t s, PITCH_PARAM unsigned int Nx, unsigned int Ny, unsigned int Nz,
                unsigned int step, double dt, double* u, double* uo, double* Lu) {
  adv_compat::note(adv_ref_rk(ADV_F64, 3, 3, PITCH_VALUE, Nx, Ny, Nz, (int)step, dt, u, uo, Lu, s), "Call_sspRK");
}

int adv_compat_last_status(void) { return adv_compat::take_status(); }
void adv_compat_set_bug_b2(int on) { g_bug_b2.store(on ? 1 : 0); }

}  // extern "C"
