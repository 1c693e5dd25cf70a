/*
 * advdiff_compat_heat3d.h -- the reference's 3D heat launch wrappers, exported with their own
 * names and signatures (REAL = double) by libadvdiff_compat_heat3d.so, so the reference's
 * SingleGPU/Diffusion3d_baselineCode/main.cpp links against this library unchanged.
 * Define ADV_COMPAT_PITCHED for the pitched signatures of SingleGPU/Diffusion3d_PitchedMem
 * (libadvdiff_compat_heat3d_pitched.so), ADV_COMPAT_BLOCKING for SingleGPU/Diffusion3d_Blocking
 * (libadvdiff_compat_heat3d_blocking.so: the same pitched signatures, acoustics3d.h:58-60; its
 * Call_Lu3d writes i, j in [3, n-4] and k in [3, nz-3], kernels.cu:37-88 and 167-171).
 *
 *   CopyToConstantMemory <- acoustics3d.h:57 (kernels.cu:147-152)
 *   Call_Lu3d            <- acoustics3d.h:58 (kernels.cu:154-158): O4 Laplacian, nodes 2..n-3
 *   Call_RK3d            <- acoustics3d.h:59 (kernels.cu:160-164): SSP-RK3 stage, nodes 2..n-3
 *
 * The launch geometry arguments are accepted and ignored (the library sizes its own grid).
 * The constants are kept by this library instead of in __constant__ memory. Errors do not
 * exit the process: they are recorded for adv_compat_last_status()/adv_last_error_string().
 */
#ifndef ADVDIFF_COMPAT_HEAT3D_H
#define ADVDIFF_COMPAT_HEAT3D_H
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif
void CopyToConstantMemory(double kx, double ky, double kz);
#if !defined(ADV_COMPAT_PITCHED) && !defined(ADV_COMPAT_BLOCKING)
void Call_Lu3d(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int nx, unsigned int ny,
               unsigned int nz, double* u, double* Lu);
void Call_RK3d(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int step, unsigned int nx,
               unsigned int ny, unsigned int nz, double dt, double* u, double* uo, double* Lu);
#else
void Call_Lu3d(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int pitch, unsigned int nx,
               unsigned int ny, unsigned int nz, double* u, double* Lu);
void Call_RK3d(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int step, unsigned int pitch,
               unsigned int nx, unsigned int ny, unsigned int nz, double dt, double* u, double* uo, double* Lu);
#endif
/* First non-OK status seen by a wrapper since the last call (then reset); 0 = ADV_OK. */
int adv_compat_last_status(void);
#ifdef __cplusplus
}
#endif
#endif
