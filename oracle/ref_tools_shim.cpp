// ref_tools_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// C entry points over the reference's host tools (SingleGPU/*/tools.cpp: the initial conditions
// and the result.bin writer). oracle/ref_build.py compiles this file together with the
// reference's tools.cpp, from where it lies, into oracle/_ref/libref_tools_<name>.so, so the
// tests can compare the library's initial conditions and result.bin with the reference's own.
// Exactly one of REF_HEAT3D, REF_HEAT2D, REF_BURGERS3D selects the program.

#if defined(REF_HEAT3D)
#include "acoustics3d.h"
extern "C" void ref_init(int ic, double* u, double dx, double dy, double dz, unsigned nx, unsigned ny,
                         unsigned nz) {
  Call_Init3D(ic, u, dx, dy, dz, nx, ny, nz);  // SingleGPU/Diffusion3d_baselineCode/tools.cpp:92
}
extern "C" void ref_save_binary(double* u, unsigned nx, unsigned ny, unsigned nz) {
  SaveBinary3D(u, nx, ny, nz);  // tools.cpp:59, writes result.bin in the working directory
}
#elif defined(REF_HEAT2D)
#include "diffusion2d.h"
extern "C" void ref_init(int ic, double* u, double dx, double dy, double, unsigned nx, unsigned ny, unsigned) {
  Call_Init2d(ic, u, dx, dy, nx, ny);  // SingleGPU/Diffusion2d/tools.cpp
}
extern "C" void ref_save_binary(double* u, unsigned nx, unsigned ny, unsigned) { SaveBinary2D(u, nx, ny); }
#elif defined(REF_BURGERS3D)
#include "Burgers.h"
extern "C" void ref_init(int ic, double* u, double dx, double dy, double dz, unsigned nx, unsigned ny,
                         unsigned nz) {
  Call_Init3d(ic, u, dx, dy, dz, nx, ny, nz);  // SingleGPU/Burgers3d_WENO5/tools.cpp
}
extern "C" void ref_save_binary(double* u, unsigned nx, unsigned ny, unsigned nz) {
  SaveBinary3D(u, nx, ny, nz);
}
#else
#error "define REF_HEAT3D, REF_HEAT2D or REF_BURGERS3D"
#endif
