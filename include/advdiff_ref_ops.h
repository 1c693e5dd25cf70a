/*
 * advdiff_ref_ops.h -- the reference's unfused operators with their exact update rules,
 * constants passed explicitly (no process-global state). Implemented in libadvdiff.so.
 *
 * These mirror the reference's per-operator launch wrappers one for one, so a caller that
 * drives its own loop (as the reference's main.cpp does) gets identical semantics, including
 * which nodes each operator touches, assignment vs accumulation into Lu, and the zero left
 * face at the start of each Burgers sweep. The compatibility libraries
 * (advdiff_compat_*.h) forward the reference's extern "C" names here.
 *
 * `pitch` is the row stride in elements (nx for dense arrays; the pitched reference variants
 * pass cudaMallocPitch's pitch / sizeof(REAL)). All buffers are device pointers.
 */
#ifndef ADVDIFF_REF_OPS_H
#define ADVDIFF_REF_OPS_H

#include <stdint.h>

#include "advdiff.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Laplacian into Lu on nodes with every index in [lo, n-lo):
 *   order 4: Lu = kx(-u[i+2]+16u[i+1]-30u+16u[i-1]-u[i-2]) + ky(..) + kz(..)
 *            (SingleGPU/Diffusion3d_baselineCode/kernels.cu:66-99, lo = 2;
 *             SingleGPU/Diffusion2d/kernels.cu:70-88, lo = 3 with zero_outside = 1)
 *   order 2: Lu = 12kx(u[i+1]-2u+u[i-1]) + ... (kernels.cu:37-64)
 * zero_outside = 1 writes Lu = 0 on every other node (the 2D kernel's else branch). */
adv_status adv_ref_laplace(int dtype, int ndim, int order, int lo, int zero_outside, int64_t pitch, int nx, int ny,
                           int nz, double kx, double ky, double kz, const void* u, void* Lu, void* stream);

/* Laplacian into Lu on the nodes of a box: box = {i0, i1, j0, j1, k0, k1}, i in [i0, i1) and so
 * on (k ignored in 2D), the same arithmetic as adv_ref_laplace; zero_outside = 1 writes Lu = 0 on
 * every other node. west_first = 1 takes the 3D O4 operands west/south/bottom first (the 2D
 * kernel's order, which SingleGPU/Diffusion3d_Blocking/kernels.cu:66-68 uses in 3D); 0 the
 * baseline's east-first order. The box must keep the stencil on the grid (i0 >= order/2,
 * i1 <= nx - order/2, ...). SingleGPU/Diffusion3d_Blocking/kernels.cu:37-88 writes i, j in
 * [3, n-4] and k in [3, nz-3] (kstart 3, kstop nz-2): box {3, nx-3, 3, ny-3, 3, nz-2}. */
adv_status adv_ref_laplace_box(int dtype, int ndim, int order, const int32_t* box, int zero_outside, int west_first,
                               int64_t pitch, int nx, int ny, int nz, double kx, double ky, double kz, const void* u,
                               void* Lu, void* stream);

/* SSP-RK3 stage `step` (1..3) in place on nodes with every index in [lo, n-lo):
 * u = uo + dt Lu | 0.75 uo + 0.25 (u + dt Lu) | (uo + 2 (u + dt Lu)) / 3
 * (SingleGPU/Diffusion3d_baselineCode/kernels.cu:104-142; Burgers kernels.cu:499-530, lo = 3). */
adv_status adv_ref_rk(int dtype, int ndim, int lo, int64_t pitch, int nx, int ny, int nz, int step, double dt,
                      void* u, const void* uo, const void* Lu, void* stream);

/* One directional WENO sweep with the reference's local Lax-Friedrichs split
 * (SingleGPU/Burgers3d_WENO5/kernels.cu:197-394): along `axis` (0 = x, 1 = y, 2 = z) on nodes
 * whose other two indices lie in [3, n-4] and whose own index runs 2..n-4; the face flux left of
 * index 2 is taken as 0, as the reference's sweeps start with fu_old = 0.
 * axis 0 assigns Lu = -(F+ - F-)/h; axes 1 and 2 subtract (F+ - F-)/h from Lu. */
adv_status adv_ref_burgers_sweep(int dtype, int axis, int weno, int64_t pitch, int nx, int ny, int nz, double h,
                                 const void* u, void* Lu, void* stream);

/* The shared-memory program's directional sweep (SingleGPU/Burgers3d_WENO5_SharedMem/
 * kernels.cu:212-405): on every node of every line along `axis`, Lu = -(F(a+1/2) - F(a-1/2))/h
 * (x: assigned; y, z: subtracted), the face flux F(a-1/2) reconstructed from nodes a-3 .. a+2 with
 * u taken as 0 beyond both ends of the line (its Dirichlet zero fill, kernels.cu:247-259), the
 * same local Lax-Friedrichs split as adv_ref_burgers_sweep and its weights normalised by a
 * reciprocal (alphasum = 1/(a0+a1+a2), times (1/6) alphasum: kernels.cu:119-129). Lu on the last
 * three nodes of a line (a > n-4) depends in the reference on shared memory its tiles never load;
 * here it takes the zero extension. Its RK stage reads none of them. */
adv_status adv_ref_burgers_sweep_all(int dtype, int axis, int weno, int64_t pitch, int nx, int ny, int nz, double h,
                                     const void* u, void* Lu, void* stream);

/* Viscous term Lu += O4 Laplacian (kx,ky,kz = C/(12 h^2)) on i,j in [3, n-4], k in [3, nz-3]
 * (SingleGPU/Burgers3d_WENO5/kernels.cu:444-494 with kstart 3, kstop nz-2, 16-slab blocks).
 * bug_b2 = 1 adds slabs 16..min(18, nz-3) twice, as the reference's overlapping z-blocks do. */
adv_status adv_ref_burgers_viscous(int dtype, int64_t pitch, int nx, int ny, int nz, double kx, double ky, double kz,
                                   int bug_b2, const void* u, void* Lu, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ADVDIFF_REF_OPS_H */
