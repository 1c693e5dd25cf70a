/*
 * advdiff_compat_burgers3d.h -- the reference's 3D Burgers launch wrappers (REAL = double),
 * exported by libadvdiff_compat_burgers3d.so so SingleGPU/Burgers3d_WENO5/main.cpp links
 * unchanged. Define ADV_COMPAT_PITCHED for SingleGPU/Burgers3d_WENO5_PitchedMem's signatures
 * (libadvdiff_compat_burgers3d_pitched.so). libadvdiff_compat_burgers3d_sharedmem.so has the same
 * pitched signatures for SingleGPU/Burgers3d_WENO5_SharedMem (Burgers.h:79-83), its Call_Adv_*
 * being that program's sweeps (adv_ref_burgers_sweep_all: every node, zero beyond the grid,
 * reciprocal weight normalisation; kernels.cu:212-405, 552-568); its Call_Diff_ and Call_sspRK are
 * the baseline's (the kernels are the same, kernels.cu:453-543).
 *
 *   CopyToConstantMemory <- Burgers.h:72 (kernels.cu:535-540): viscous constants C/(12 h^2)
 *   Call_Adv_x           <- Burgers.h:73 (kernels.cu:542-546): Lu  = -dF/dx (WENO5-Z, local LF)
 *   Call_Adv_y           <- Burgers.h:75 (kernels.cu:548-552): Lu -= dG/dy
 *   Call_Adv_z           <- Burgers.h:77 (kernels.cu:554-558): Lu -= dH/dz
 *   Call_Diff_           <- Burgers.h:79 (kernels.cu:560-565): Lu += viscous O4 term; slabs
 *                           16..18 are added twice as the reference's z-blocks do, unless
 *                           adv_compat_set_bug_b2(0) was called
 *   Call_sspRK           <- Burgers.h:81 (kernels.cu:567-571): SSP-RK3 stage on nodes 3..n-4
 *
 * Launch geometry arguments are accepted and ignored (the reference's swapped x/y sweep grids,
 * SingleGPU/Burgers3d_WENO5/main.cpp:101,105, therefore do not truncate non-cubic runs here).
 */
#ifndef ADVDIFF_COMPAT_BURGERS3D_H
#define ADVDIFF_COMPAT_BURGERS3D_H
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif
void CopyToConstantMemory(double kx, double ky, double kz);
#ifndef ADV_COMPAT_PITCHED
void Call_Adv_x(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int Nx, unsigned int Ny,
                unsigned int Nz, double dx, double* u, double* Lu);
void Call_Adv_y(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int Nx, unsigned int Ny,
                unsigned int Nz, double dy, double* v, double* Lv);
void Call_Adv_z(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int Nx, unsigned int Ny,
                unsigned int Nz, double dz, double* w, double* Lw);
void Call_Diff_(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int Nx, unsigned int Ny,
                unsigned int Nz, double* q, double* Lq);
void Call_sspRK(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int Nx, unsigned int Ny,
                unsigned int Nz, unsigned int step, double dt, double* u, double* uo, double* Lu);
#else
void Call_Adv_x(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int pitch, unsigned int Nx,
                unsigned int Ny, unsigned int Nz, double dx, double* u, double* Lu);
void Call_Adv_y(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int pitch, unsigned int Nx,
                unsigned int Ny, unsigned int Nz, double dy, double* v, double* Lv);
void Call_Adv_z(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int pitch, unsigned int Nx,
                unsigned int Ny, unsigned int Nz, double dz, double* w, double* Lw);
void Call_Diff_(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int pitch, unsigned int Nx,
                unsigned int Ny, unsigned int Nz, double* q, double* Lq);
void Call_sspRK(dim3 numBlocks, dim3 threadsPerBlock, cudaStream_t aStream, unsigned int pitch, unsigned int Nx,
                unsigned int Ny, unsigned int Nz, unsigned int step, double dt, double* u, double* uo, double* Lu);
#endif
int adv_compat_last_status(void);
/* 1 (default): reproduce the reference's doubled viscous slabs 16..18; 0: add them once. */
void adv_compat_set_bug_b2(int on);
#ifdef __cplusplus
}
#endif
#endif
