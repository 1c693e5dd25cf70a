/*
 * advdiff_compat_heat2d.h -- the reference's 2D heat launch wrappers (REAL = double), exported
 * by libadvdiff_compat_heat2d.so so SingleGPU/Diffusion2d/main.cpp links unchanged.
 * Define ADV_COMPAT_PITCHED for SingleGPU/Diffusion2d_PitchedMem's signatures
 * (libadvdiff_compat_heat2d_pitched.so).
 *
 *   CopyToConstantMemory <- diffusion2d.h:57 (kernels.cu:155-159)
 *   Call_Lu2d            <- diffusion2d.h:58 (kernels.cu:161-165): O4 Laplacian on nodes 3..n-4,
 *                           Lu = 0 elsewhere
 *   Call_RK2d            <- diffusion2d.h:59 (kernels.cu:167-171): SSP-RK3 stage on nodes 3..n-4
 *
 * Launch geometry arguments are accepted and ignored; errors are recorded, never exit.
 */
#ifndef ADVDIFF_COMPAT_HEAT2D_H
#define ADVDIFF_COMPAT_HEAT2D_H
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif
void CopyToConstantMemory(const double kx, const double ky);
#ifndef ADV_COMPAT_PITCHED
void Call_Lu2d(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int nx, unsigned int ny, double* u,
               double* Lu);
void Call_RK2d(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int step, unsigned int nx,
               unsigned int ny, double dt, double* u, double* uo, double* Lu);
#else
void Call_Lu2d(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int pitch, unsigned int nx,
               unsigned int ny, double* u, double* Lu);
void Call_RK2d(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int step, unsigned int pitch,
               unsigned int nx, unsigned int ny, double dt, double* u, double* uo, double* Lu);
#endif
int adv_compat_last_status(void);
#ifdef __cplusplus
}
#endif
#endif
