// advdiff_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference's numerical schemes for the two explicit solvers
// (heat-equation stencil + time update, 3D Burgers WENO5/WENO5-Z + Lax-Friedrichs + SSP-RK3).
// It is the parity oracle for the CUDA path and the timed CPU baseline. Only the tests,
// the smoke check and the CPU-baseline leg of the benchmark load this library; the product
// library never links, calls or falls back to it.
//
// FP64 is the reference's own precision (SingleGPU/Burgers3d_WENO5/Burgers.h:47-54,
// SingleGPU/Diffusion3d_baselineCode/acoustics3d.h:35-42). Every routine is templated on the
// arithmetic type so an FP32 variant can measure the single-precision error floor on the CPU.
//
// Parity pins (checked by tests/test_oracle_golden.py):
//   * Matlab_Prototipes/DiffusionNd/TestingAccuracy.log:53-72 (O4 + SSP-RK3 heat 1D/2D/3D),
//     reproduced by orc_heat_accuracy() which follows diffusion{1,2,3}dTest.m literally, and
//     the same functions run through an interpreter for their MATLAB subset (full precision);
//   * recorded "Final Time" 0.325 / 0.329157 (SingleGPU/Diffusion2d/Run.m:11,
//     SingleGPU/Diffusion3d_baselineCode/Run.m:11) via the reference dt rule;
//   * recorded iteration counts 86 / 167 / 267 of the Burgers dt loop
//     (SingleGPU/Burgers3d_WENO5/Run.m:24,36; SingleGPU/Burgers3d_WENO5_Hybrid2/Run.m:12);
//   * the MATLAB Burgers prototypes (WENO5 / WENO7 residuals and solver loops of
//     Matlab_Prototipes/InviscidBurgersNd), whose outputs were produced by running those .m
//     files through an interpreter for their MATLAB subset (tests/test_oracle_prototypes.py).
//
// Built with -ffp-contract=off so x86 and Arm hosts give bitwise identical results.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ------------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11). Counter-based; used for every seeded synthetic input.
// ------------------------------------------------------------------------------------------
inline void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Two uniforms in [0,1) with 53-bit resolution from draw `idx` of stream `stream`.
inline void philox_u01x2(uint32_t seed, uint32_t stream, uint64_t idx, double* a, double* b) {
  uint32_t ctr[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 0u, 0u};
  uint32_t key[2] = {seed, stream};
  uint32_t o[4];
  philox4x32_10(ctr, key, o);
  const double s = 1.0 / 9007199254740992.0;  // 2^-53
  *a = (double)(((uint64_t)o[0] << 21) ^ (uint64_t)(o[1] >> 11)) * s;
  *b = (double)(((uint64_t)o[2] << 21) ^ (uint64_t)(o[3] >> 11)) * s;
}

inline int64_t wrap(int64_t i, int64_t n) { i %= n; return i < 0 ? i + n : i; }

// ------------------------------------------------------------------------------------------
// Heat: one fused stage. Laplacian as SingleGPU/Diffusion3d_baselineCode/kernels.cu:37-99
// (O2 7-pt / O4 13-pt, same operand order), 2D as SingleGPU/Diffusion2d/kernels.cu:70-88,
// stage update as kernels.cu:104-142 (stage 1 == forward Euler).
//   order:   2 -> k*(e - 2o + w) per axis; 4 -> k*(-ee + 16e - 30o + 16w - ww) per axis.
//   frozen:  outer layers that are never updated (copied through); the reference freezes
//            2 layers in 3D (kernels.cu:127) and 3 in 2D (Diffusion2d/kernels.cu:53).
//   zero_boundary: the outermost layer is written as 0 (Dirichlet u=0).
//   periodic: every node is updated and neighbours wrap.
// ------------------------------------------------------------------------------------------
struct HeatCfg {
  int ndim, nx, ny, nz, order, frozen, zero_boundary, periodic;
  double kx, ky, kz, dt;
};

template <class T>
inline T stage_combine(int stage, T un, T uin, T dt, T L) {
  switch (stage) {
    case 2: return (T)0.75 * un + (T)0.25 * (uin + dt * L);
    case 3: return (un + (T)2 * (uin + dt * L)) / (T)3;
    default: return un + dt * L;
  }
}

template <class T>
void heat_stage(const HeatCfg& c, int stage, const T* uin, const T* un, T* out) {
  const int64_t nx = c.nx, ny = c.ny, nz = (c.ndim == 3) ? c.nz : 1;
  const int64_t sx = 1, sy = nx, sz = nx * ny;
  const T kx = (T)c.kx, ky = (T)c.ky, kz = (T)c.kz, dt = (T)c.dt;
  const int F = c.periodic ? 0 : c.frozen;
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t k = 0; k < nz; ++k)
    for (int64_t j = 0; j < ny; ++j)
      for (int64_t i = 0; i < nx; ++i) {
        const int64_t o = i + nx * j + sz * k;
        bool interior = i >= F && i < nx - F && j >= F && j < ny - F;
        if (c.ndim == 3) interior = interior && k >= F && k < nz - F;
        if (!interior) {
          bool outer = i == 0 || i == nx - 1 || j == 0 || j == ny - 1;
          if (c.ndim == 3) outer = outer || k == 0 || k == nz - 1;
          out[o] = (c.zero_boundary && outer) ? (T)0 : uin[o];
          continue;
        }
        auto at = [&](int64_t di, int64_t dj, int64_t dk) -> T {
          if (c.periodic)
            return uin[wrap(i + di, nx) + nx * wrap(j + dj, ny) + sz * wrap(k + dk, nz)];
          return uin[o + di * sx + dj * sy + dk * sz];
        };
        const T uo = uin[o];
        T L;
        if (c.order == 4 && c.ndim == 2) {
          // 2D operand order is west/south first (SingleGPU/Diffusion2d/kernels.cu:82-83).
          T Sx = -at(-2, 0, 0) + (T)16 * at(-1, 0, 0) - (T)30 * uo + (T)16 * at(1, 0, 0) - at(2, 0, 0);
          T Sy = -at(0, -2, 0) + (T)16 * at(0, -1, 0) - (T)30 * uo + (T)16 * at(0, 1, 0) - at(0, 2, 0);
          L = kx * Sx + ky * Sy;
        } else if (c.order == 4) {
          // 3D operand order is east/north/top first (Diffusion3d_baselineCode/kernels.cu:95-97).
          T Sx = -at(2, 0, 0) + (T)16 * at(1, 0, 0) - (T)30 * uo + (T)16 * at(-1, 0, 0) - at(-2, 0, 0);
          T Sy = -at(0, 2, 0) + (T)16 * at(0, 1, 0) - (T)30 * uo + (T)16 * at(0, -1, 0) - at(0, -2, 0);
          L = kx * Sx + ky * Sy;
          if (c.ndim == 3) {
            T Sz = -at(0, 0, 2) + (T)16 * at(0, 0, 1) - (T)30 * uo + (T)16 * at(0, 0, -1) - at(0, 0, -2);
            L = L + kz * Sz;
          }
        } else {
          T Sx = at(1, 0, 0) - (T)2 * uo + at(-1, 0, 0);
          T Sy = at(0, 1, 0) - (T)2 * uo + at(0, -1, 0);
          L = kx * Sx + ky * Sy;
          if (c.ndim == 3) {
            T Sz = at(0, 0, 1) - (T)2 * uo + at(0, 0, -1);
            L = L + kz * Sz;
          }
        }
        out[o] = stage_combine<T>(stage, un[o], uo, dt, L);
      }
}

// The GPU path's fused multiply-add evaluation order (FP32 always, FP64 with the descriptor's
// `contract`; see the product's heat_stage.cuh). Mathematically the same stencil and stage update
// as heat_stage(); used to check those kernels bit for bit.
//   O2 per axis: fma(-2, c, p1) + m1;  O4 per axis: fma(16, far1, fma(-30, c, fma(16, near1,
//   -near2))) - far2 with near = +1 in 3D and -1 in 2D;  L = fma(kz, Sz, fma(ky, Sy, kx*Sx));
//   stages: fma(dt, L, un) | fma(0.25, fma(dt, L, uin), 0.75*un) | fma(2, fma(dt, L, uin), un)/3.
template <class T>
void heat_stage_fma(const HeatCfg& c, int stage, const T* uin, const T* un, T* out) {
  const int64_t nx = c.nx, ny = c.ny, nz = (c.ndim == 3) ? c.nz : 1;
  const int64_t sz = nx * ny;
  const T kx = (T)c.kx, ky = (T)c.ky, kz = (T)c.kz, dt = (T)c.dt;
  const int F = c.frozen;
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t k = 0; k < nz; ++k)
    for (int64_t j = 0; j < ny; ++j)
      for (int64_t i = 0; i < nx; ++i) {
        const int64_t o = i + nx * j + sz * k;
        bool interior = i >= F && i < nx - F && j >= F && j < ny - F;
        if (c.ndim == 3) interior = interior && k >= F && k < nz - F;
        if (!interior) {
          bool outer = i == 0 || i == nx - 1 || j == 0 || j == ny - 1;
          if (c.ndim == 3) outer = outer || k == 0 || k == nz - 1;
          out[o] = (c.zero_boundary && outer) ? T(0) : uin[o];
          continue;
        }
        const T ce = uin[o];
        auto axis = [&](int64_t s) -> T {
          const T p1 = uin[o + s], m1 = uin[o - s];
          if (c.order == 2) return std::fma(T(-2), ce, p1) + m1;
          const T p2 = uin[o + 2 * s], m2 = uin[o - 2 * s];
          const bool plus_first = c.ndim == 3;
          const T a1 = plus_first ? p1 : m1, a2 = plus_first ? p2 : m2;
          const T b1 = plus_first ? m1 : p1, b2 = plus_first ? m2 : p2;
          return std::fma(T(16), b1, std::fma(T(-30), ce, std::fma(T(16), a1, -a2))) - b2;
        };
        T L = std::fma(ky, axis(nx), kx * axis(1));
        if (c.ndim == 3) L = std::fma(kz, axis(sz), L);
        T v;
        if (stage == 2) v = std::fma(T(0.25), std::fma(dt, L, ce), T(0.75) * un[o]);
        else if (stage == 3) v = std::fma(T(2), std::fma(dt, L, ce), un[o]) / T(3);
        else v = std::fma(dt, L, un[o]);
        out[o] = v;
      }
}

template <class T>
void heat_run_fma(const HeatCfg& c, int time, int64_t nsteps, T* u) {
  const size_t n = (size_t)c.nx * c.ny * (c.ndim == 3 ? c.nz : 1);
  std::vector<T> a(n), b(n);
  for (int64_t s = 0; s < nsteps; ++s) {
    heat_stage_fma<T>(c, 1, u, u, a.data());
    if (time != 0) {
      heat_stage_fma<T>(c, 2, a.data(), u, b.data());
      heat_stage_fma<T>(c, 3, b.data(), u, a.data());
    }
    std::memcpy(u, a.data(), n * sizeof(T));
  }
}

// Fixed-step run: `time`==0 forward Euler, `time`==1 SSP-RK3 (the reference's heat loop,
// SingleGPU/Diffusion3d_baselineCode/main.cpp:106-122). Result left in u.
template <class T>
void heat_run(const HeatCfg& c, int time, int64_t nsteps, T* u) {
  const size_t n = (size_t)c.nx * c.ny * (c.ndim == 3 ? c.nz : 1);
  std::vector<T> a(n), b(n);
  for (int64_t s = 0; s < nsteps; ++s) {
    if (time == 0) {
      heat_stage<T>(c, 1, u, u, a.data());
      std::memcpy(u, a.data(), n * sizeof(T));
    } else {
      heat_stage<T>(c, 1, u, u, a.data());
      heat_stage<T>(c, 2, a.data(), u, b.data());
      heat_stage<T>(c, 3, b.data(), u, a.data());
      std::memcpy(u, a.data(), n * sizeof(T));
    }
  }
}

// The z-blocked heat program's loop (SingleGPU/Diffusion3d_Blocking/main.cpp:101-123): Lu zeroed
// once; per SSP-RK3 stage the O4 Laplacian on i, j in [3, n-4] and k in
// [3, nz-3] (kernels.cu:37-88 with kstart 3, kstop nz-2, wrappers :167-171), then the stage update
// in place on every index in [2, n-3] (kernels.cu:93-126). Nodes of the update range outside the
// Laplacian's keep Lu = 0.
template <class T>
void heat_blocking_run(int64_t nx, int64_t ny, int64_t nz, T kx, T ky, T kz, T dt, int64_t iters, T* u) {
  const int64_t sz = nx * ny, n = sz * nz;
  std::vector<T> uo(n), Lu(n, (T)0);
  for (int64_t it = 0; it < iters; ++it) {
    std::memcpy(uo.data(), u, n * sizeof(T));
    for (int stage = 1; stage <= 3; ++stage) {
#pragma omp parallel for collapse(2) schedule(static)
      for (int64_t k = 3; k < nz - 2; ++k)
        for (int64_t j = 3; j < ny - 3; ++j)
          for (int64_t i = 3; i < nx - 3; ++i) {
            const int64_t o = i + nx * j + sz * k;
            const T c = u[o];
            // west/south/bottom first (kernels.cu:66-68, 78-80), unlike the baseline's 3D kernel
            T Sx = -u[o - 2] + (T)16 * u[o - 1] - (T)30 * c + (T)16 * u[o + 1] - u[o + 2];
            T Sy = -u[o - 2 * nx] + (T)16 * u[o - nx] - (T)30 * c + (T)16 * u[o + nx] - u[o + 2 * nx];
            T Sz = -u[o - 2 * sz] + (T)16 * u[o - sz] - (T)30 * c + (T)16 * u[o + sz] - u[o + 2 * sz];
            Lu[o] = kx * Sx + ky * Sy + kz * Sz;
          }
#pragma omp parallel for collapse(2) schedule(static)
      for (int64_t k = 2; k < nz - 2; ++k)
        for (int64_t j = 2; j < ny - 2; ++j)
          for (int64_t i = 2; i < nx - 2; ++i) {
            const int64_t o = i + nx * j + sz * k;
            u[o] = stage_combine<T>(stage, uo[o], u[o], dt, Lu[o]);
          }
    }
  }
}

// ------------------------------------------------------------------------------------------
// Burgers. Flux f = u^2/2 (SingleGPU/Burgers3d_WENO5/kernels.cu:37-40), Lax-Friedrichs split
// f+- = (f +- a u)/2 (kernels.cu:224-238; a = |u| local, or a = max|u| global as in
// Matlab_Prototipes/InviscidBurgersNd/LFWENO5FDM3d.m:71 with a scalar). Face flux
// F_{i+1/2} = WENO(f+ at i-2..i+2) + WENO(f- at i-1..i+3): WENO5-Z as kernels.cu:142-192,
// WENO5-JS as kernels.cu:92-140 (= MultiGPU/Burgers3d_Baseline/Kernels.cu:112-222).
// The divisions of the smoothness-indicator weights run in type D.
// ------------------------------------------------------------------------------------------
// recip: the shared-memory program's normalisation (SingleGPU/Burgers3d_WENO5_SharedMem/
// kernels.cu:119-129, 143-146): alphasum = 1/(a0+a1+a2), the weighted sum times (1/6)*alphasum.
template <class T, class D>
inline T weno_face(int z, T vmm, T vm, T v, T vp, T vpp, T umm, T um, T u, T up, T upp, int recip = 0) {
  const T c1312 = (T)(13. / 12.), c14 = (T)(1. / 4.);
  const D eps = (D)1e-6;
  T B0 = c1312 * (vmm - (T)2 * vm + v) * (vmm - (T)2 * vm + v) + c14 * (vmm - (T)4 * vm + (T)3 * v) * (vmm - (T)4 * vm + (T)3 * v);
  T B1 = c1312 * (vm - (T)2 * v + vp) * (vm - (T)2 * v + vp) + c14 * (vm - vp) * (vm - vp);
  T B2 = c1312 * (v - (T)2 * vp + vpp) * (v - (T)2 * vp + vpp) + c14 * ((T)3 * v - (T)4 * vp + vpp) * ((T)3 * v - (T)4 * vp + vpp);
  D a0, a1, a2;
  if (z) {
    D tau5 = std::fabs((D)B0 - (D)B2);
    a0 = (D)(1. / 10.) * ((D)1 + tau5 / ((D)B0 + eps));
    a1 = (D)(6. / 10.) * ((D)1 + tau5 / ((D)B1 + eps));
    a2 = (D)(3. / 10.) * ((D)1 + tau5 / ((D)B2 + eps));
  } else {
    a0 = (D)(1. / 10.) / ((eps + (D)B0) * (eps + (D)B0));
    a1 = (D)(6. / 10.) / ((eps + (D)B1) * (eps + (D)B1));
    a2 = (D)(3. / 10.) / ((eps + (D)B2) * (eps + (D)B2));
  }
  D asum = a0 + a1 + a2;
  auto normalise = [&](D num, D sum) { return recip ? num * ((D)(1. / 6.) * ((D)1 / sum)) : num / ((D)6 * sum); };
  D fm = normalise(a0 * (D)((T)2 * vmm - (T)7 * vm + (T)11 * v) + a1 * (D)(-vm + (T)5 * v + (T)2 * vp) +
                       a2 * (D)((T)2 * v + (T)5 * vp - vpp),
                   asum);

  B0 = c1312 * (umm - (T)2 * um + u) * (umm - (T)2 * um + u) + c14 * (umm - (T)4 * um + (T)3 * u) * (umm - (T)4 * um + (T)3 * u);
  B1 = c1312 * (um - (T)2 * u + up) * (um - (T)2 * u + up) + c14 * (um - up) * (um - up);
  B2 = c1312 * (u - (T)2 * up + upp) * (u - (T)2 * up + upp) + c14 * ((T)3 * u - (T)4 * up + upp) * ((T)3 * u - (T)4 * up + upp);
  if (z) {
    D tau5 = std::fabs((D)B0 - (D)B2);
    a0 = (D)(3. / 10.) * ((D)1 + tau5 / ((D)B0 + eps));
    a1 = (D)(6. / 10.) * ((D)1 + tau5 / ((D)B1 + eps));
    a2 = (D)(1. / 10.) * ((D)1 + tau5 / ((D)B2 + eps));
  } else {
    a0 = (D)(3. / 10.) / ((eps + (D)B0) * (eps + (D)B0));
    a1 = (D)(6. / 10.) / ((eps + (D)B1) * (eps + (D)B1));
    a2 = (D)(1. / 10.) / ((eps + (D)B2) * (eps + (D)B2));
  }
  asum = a0 + a1 + a2;
  D fp = normalise(a0 * (D)(-umm + (T)5 * um + (T)2 * u) + a1 * (D)((T)2 * um + (T)5 * u - up) +
                       a2 * (D)((T)11 * u - (T)7 * up + (T)2 * upp),
                   asum);
  return (T)fm + (T)fp;
}

struct BurgersCfg {
  int nx, ny, nz;
  int weno_z;     // 1: WENO5-Z, 0: WENO5-JS
  int lf_global;  // 1: a = max|u| of the stage input, 0: a = |u| per node
  int periodic;   // 1: periodic wrap; 0: reference frozen boundary (3 layers)
  int bug_b2;     // reproduce the doubled viscous slabs 16..18 of the reference
  double dx, dy, dz;
  double kx, ky, kz;  // viscous O4 coefficients C/(12 h^2); 0 disables the term
  int recip = 0;      // 1: the shared-memory program's weight normalisation (weno_face)
};

template <class T>
inline void lf_split(T u, T a_glob, int global, T* fp, T* fm) {
  T f = (T)0.5 * u * u;
  T a = global ? a_glob : std::fabs(u);
  *fp = (T)0.5 * (f + a * u);
  *fm = (T)0.5 * (f - a * u);
}

// Face flux at +1/2 of position p along an axis: cells p-2..p+3 given by `get`.
template <class T, class D, class G>
inline T face_flux(const BurgersCfg& c, T a_glob, G get) {
  T fp[6], fm[6];
  for (int q = 0; q < 6; ++q) lf_split<T>(get(q - 2), a_glob, c.lf_global, &fp[q], &fm[q]);
  return weno_face<T, D>(c.weno_z, fp[0], fp[1], fp[2], fp[3], fp[4], fm[1], fm[2], fm[3], fm[4], fm[5], c.recip);
}

// The shared-memory program's directional sweep (SingleGPU/Burgers3d_WENO5_SharedMem/
// kernels.cu:212-405) on every node of every line along `axis`: u = 0 beyond both ends of a line
// (its Dirichlet fill, kernels.cu:247-259), F(a-1/2) from nodes a-3 .. a+2 with the local split
// and the reciprocal normalisation; x assigns Lu = -(F(a+1/2) - F(a-1/2))/h, y and z subtract
// (F(a+1/2) - F(a-1/2))/h. The reference defines Lu only for a <= n-4 (its tiles leave the
// shared-memory cells past the grid unloaded); the zero extension is used for the last three.
template <class T>
void sweep_all(int axis, int weno_z, int64_t nx, int64_t ny, int64_t nz, T h, const T* u, T* Lu) {
  const int64_t na = axis == 0 ? nx : axis == 1 ? ny : nz;
  const int64_t nb = axis == 0 ? ny : nx, nc = axis == 2 ? ny : nz;
  const int64_t s = axis == 0 ? 1 : axis == 1 ? nx : nx * ny;
  BurgersCfg c{};
  c.weno_z = weno_z;
  c.recip = 1;
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < nb * nc; ++t) {
    const int64_t b = t % nb, cc = t / nb;
    const int64_t i = axis == 0 ? 0 : b, j = axis == 0 ? b : (axis == 1 ? 0 : cc), k = axis == 2 ? 0 : cc;
    const int64_t o0 = i + nx * j + nx * ny * k;
    auto get = [&](int64_t a) -> T { return a >= 0 && a < na ? u[o0 + a * s] : (T)0; };
    for (int64_t a = 0; a < na; ++a) {
      const T fr = face_flux<T, T>(c, (T)0, [&](int q) { return get(a + q); });
      const T fl = face_flux<T, T>(c, (T)0, [&](int q) { return get(a - 1 + q); });
      const int64_t o = o0 + a * s;
      if (axis == 0) Lu[o] = -(fr - fl) / h;
      else Lu[o] = Lu[o] - (fr - fl) / h;
    }
  }
}

// Right-hand side Lu at every updated cell (others untouched). Accumulation order follows
// the reference's sweeps: Lu = -(dF)/dx; Lu -= dG/dy; Lu -= dH/dz; Lu += viscous
// (SingleGPU/Burgers3d_WENO5/main.cpp:143-149; kernels.cu:197-494).
template <class T, class D>
void burgers_rhs(const BurgersCfg& c, const T* u, T a_glob, T* Lu) {
  const int64_t nx = c.nx, ny = c.ny, nz = c.nz, sz = nx * ny;
  const int F = c.periodic ? 0 : 3;
  const int Fz = nz == 1 ? 0 : F;  // 2D (one plane): no frozen z layers, z neighbours are the plane
  const T dx = (T)c.dx, dy = (T)c.dy, dz = (T)c.dz;
  const T kx = (T)c.kx, ky = (T)c.ky, kz = (T)c.kz;
  const bool visc = c.kx != 0.0 || c.ky != 0.0 || c.kz != 0.0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t k = Fz; k < nz - Fz; ++k)
    for (int64_t j = F; j < ny - F; ++j)
      for (int64_t i = F; i < nx - F; ++i) {
        const int64_t o = i + nx * j + sz * k;
        auto U = [&](int64_t ii, int64_t jj, int64_t kk) -> T {
          if (c.periodic) return u[wrap(ii, nx) + nx * wrap(jj, ny) + sz * wrap(kk, nz)];
          if (nz == 1) kk = 0;
          return u[ii + nx * jj + sz * kk];
        };
        T fxp = face_flux<T, D>(c, a_glob, [&](int q) { return U(i + q, j, k); });
        T fxm = face_flux<T, D>(c, a_glob, [&](int q) { return U(i - 1 + q, j, k); });
        T fyp = face_flux<T, D>(c, a_glob, [&](int q) { return U(i, j + q, k); });
        T fym = face_flux<T, D>(c, a_glob, [&](int q) { return U(i, j - 1 + q, k); });
        T fzp = face_flux<T, D>(c, a_glob, [&](int q) { return U(i, j, k + q); });
        T fzm = face_flux<T, D>(c, a_glob, [&](int q) { return U(i, j, k - 1 + q); });
        T L = -(fxp - fxm) / dx;
        L = L - (fyp - fym) / dy;
        L = L - (fzp - fzm) / dz;
        if (visc) {
          const T ce = u[o];
          T v = kx * (-U(i - 2, j, k) + (T)16 * U(i - 1, j, k) - (T)30 * ce + (T)16 * U(i + 1, j, k) - U(i + 2, j, k)) +
                ky * (-U(i, j - 2, k) + (T)16 * U(i, j - 1, k) - (T)30 * ce + (T)16 * U(i, j + 1, k) - U(i, j + 2, k)) +
                kz * (-U(i, j, k - 2) + (T)16 * U(i, j, k - 1) - (T)30 * ce + (T)16 * U(i, j, k + 1) - U(i, j, k + 2));
          L = L + v;
          // Reference bug B2: Compute_Laplace_Async's first z-block starts at max(kstart,0)=3 but
          // still runs LOOP=16 slabs, so slabs 16..18 are added twice (kernels.cu:464-491).
          if (c.bug_b2 && !c.periodic && k >= 16 && k <= 18 && k <= nz - 3) L = L + v;
        }
        Lu[o] = L;
      }
}

template <class T>
T max_abs(const T* u, size_t n) {
  T m = 0;
#pragma omp parallel for reduction(max : m) schedule(static)
  for (size_t i = 0; i < n; ++i) m = std::max(m, (T)std::fabs(u[i]));
  return m;
}

// One SSP-RK3 stage: out = combine(un, uin, dt, Lu) on updated cells, uin elsewhere.
template <class T>
void burgers_combine(const BurgersCfg& c, int stage, const T* uin, const T* un, const T* Lu, T dt, T* out) {
  const int64_t nx = c.nx, ny = c.ny, nz = c.nz;
  const int F = c.periodic ? 0 : 3;
  const int Fz = nz == 1 ? 0 : F;
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t k = 0; k < nz; ++k)
    for (int64_t j = 0; j < ny; ++j)
      for (int64_t i = 0; i < nx; ++i) {
        const int64_t o = i + nx * j + nx * ny * k;
        bool interior = i >= F && i < nx - F && j >= F && j < ny - F && k >= Fz && k < nz - Fz;
        out[o] = interior ? stage_combine<T>(stage, un[o], uin[o], dt, Lu[o]) : uin[o];
      }
}

template <class T, class D>
void burgers_stage(const BurgersCfg& c, int stage, const T* uin, const T* un, double dt, T* out, T* Lu_scratch) {
  const size_t n = (size_t)c.nx * c.ny * c.nz;
  T a = c.lf_global ? max_abs<T>(uin, n) : (T)0;
  burgers_rhs<T, D>(c, uin, a, Lu_scratch);
  burgers_combine<T>(c, stage, uin, un, Lu_scratch, (T)dt, out);
}

// Time loop. dt_rule 0: reference fixed dt = min(CFL*dx/1.0, 0.9/(2C sum 1/h^2))
// (SingleGPU/Burgers3d_WENO5/main.cpp:127-136; C from the viscous coefficient, the second
// bound dropped when C == 0). dt_rule 1: dt = CFL*dx/max|u^n| (LFWENO5FDM3d.m:71).
// Both trim the last step to hit tEnd and accumulate t in FP64.
template <class T, class D>
int64_t burgers_run(const BurgersCfg& c, T* u, double tEnd, double CFL, int dt_rule, double C,
                    int64_t max_steps, double* t_out) {
  const size_t n = (size_t)c.nx * c.ny * c.nz;
  std::vector<T> a(n), b(n), Lu(n, (T)0);
  double t = 0.0;
  int64_t it = 0;
  while (t < tEnd && it < max_steps) {
    double dt;
    if (dt_rule == 0) {
      double dt1 = CFL * c.dx / 1.0;
      const double iz = c.nz == 1 ? 0.0 : 1 / c.dz / c.dz;  // 2D: no z term
      double dt2 = (C > 0) ? 1. / (2 * C * (1 / c.dx / c.dx + 1 / c.dy / c.dy + iz)) * 0.9
                           : std::numeric_limits<double>::infinity();
      dt = dt1 < dt2 ? dt1 : dt2;
    } else {
      dt = CFL * c.dx / (double)max_abs<T>(u, n);
    }
    if ((t + dt) > tEnd) dt = tEnd - t;
    t += dt;
    it += 1;
    burgers_stage<T, D>(c, 1, u, u, dt, a.data(), Lu.data());
    burgers_stage<T, D>(c, 2, a.data(), u, dt, b.data(), Lu.data());
    burgers_stage<T, D>(c, 3, b.data(), u, dt, a.data(), Lu.data());
    std::memcpy(u, a.data(), n * sizeof(T));
  }
  if (t_out) *t_out = t;
  return it;
}

}  // namespace

// ------------------------------------------------------ heat with a diffusivity field k(x)
// Conservative 7-point form with arithmetic face averages and forward Euler, c_a = dt/h_a^2, the
// outermost layer frozen (or zeroed), and the exact transpose of one step (the library's
// adv_heatk_step / adv_heatk_adjoint_step; no reference counterpart). Every operation is rounded
// as written, fused multiply-adds where the kernels use them, so the GPU agrees bit for bit.
template <class T>
void heatk_step(int64_t nx, int64_t ny, int64_t nz, int zero_boundary, T cx, T cy, T cz, const T* k, const T* u,
                T* out) {
  const int64_t sy = nx, sz = nx * ny;
  const T h = T(0.5);
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t z = 0; z < nz; ++z)
    for (int64_t y = 0; y < ny; ++y)
      for (int64_t x = 0; x < nx; ++x) {
        const int64_t o = x + sy * y + sz * z;
        const bool in = x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < nz - 1;
        const T uc = u[o], kc = k[o];
        if (!in) {
          out[o] = zero_boundary ? T(0) : uc;
          continue;
        }
        auto flux = [&](int64_t s) {
          const T fp = h * (kc + k[o + s]), fm = h * (kc + k[o - s]);
          return std::fma(fp, u[o + s] - uc, -(fm * (uc - u[o - s])));
        };
        const T Fx = flux(1), Fy = flux(sy), Fz = flux(sz);
        out[o] = uc + std::fma(cz, Fz, std::fma(cy, Fy, cx * Fx));
      }
}

template <class T>
void heatk_adjoint(int64_t nx, int64_t ny, int64_t nz, int zero_boundary, T cx, T cy, T cz, const T* k, const T* u,
                   const T* lam, T* out, T* grad) {
  const int64_t sy = nx, sz = nx * ny;
  const T h = T(0.5);
  auto interior = [&](int64_t x, int64_t y, int64_t z) {
    return x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < nz - 1;
  };
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t z = 0; z < nz; ++z)
    for (int64_t y = 0; y < ny; ++y)
      for (int64_t x = 0; x < nx; ++x) {
        const int64_t o = x + sy * y + sz * z;
        const bool in_c = interior(x, y, z);
        const T lc = lam[o], muc = in_c ? lc : T(0), uc = u[o], kc = k[o];
        auto axis = [&](int64_t s, bool hp, bool hm, bool inp, bool inm, T& S, T& G) {
          const int64_t op = hp ? o + s : o, om = hm ? o - s : o;
          const T mup = hp && inp ? lam[op] : T(0), mum = hm && inm ? lam[om] : T(0);
          const T kfp = h * (kc + k[op]), kfm = h * (kc + k[om]);
          const T dmp = hp ? mup - muc : T(0), dmm = hm ? mum - muc : T(0);
          const T dup = u[op] - uc, dum = u[om] - uc;
          S = std::fma(kfm, dmm, kfp * dmp);
          G = std::fma(dum, -dmm, dup * -dmp);
        };
        T Sx, Gx, Sy, Gy, Sz, Gz;
        axis(1, x + 1 < nx, x > 0, interior(x + 1, y, z), interior(x - 1, y, z), Sx, Gx);
        axis(sy, y + 1 < ny, y > 0, interior(x, y + 1, z), interior(x, y - 1, z), Sy, Gy);
        axis(sz, z + 1 < nz, z > 0, interior(x, y, z + 1), interior(x, y, z - 1), Sz, Gz);
        const T keep = (in_c || !zero_boundary) ? lc : T(0);
        out[o] = keep + std::fma(cz, Sz, std::fma(cy, Sy, cx * Sx));
        grad[o] = std::fma(h, std::fma(cz, Gz, std::fma(cy, Gy, cx * Gx)), grad[o]);
      }
}

// ------------------------------------------------------------ Burgers discrete adjoint
// Exact transpose of the periodic, local Lax-Friedrichs WENO5 / WENO5-Z SSP-RK3 step (the
// library's adv_burgers_adjoint_step; no reference counterpart). Written independently of the
// kernel, in scatter form: every face pushes its derivative into the ten cells of its stencil.
//
// One side of a face from a..e (the left-biased five values); the WENO weights in their
// common-denominator form w_k (alpha_k times a positive factor shared by the three):
//   B_k = 13/3 t_k^2 + s_k^2 + 4e-6   (= 4 (beta_k + eps))
//   Z:  w_0 = (B0+tau) B1 B2, w_1 = 6 (B1+tau) B0 B2, w_2 = 3 (B2+tau) B0 B1, tau = |B0-B2|
//   JS: w_0 = (B1 B2)^2,      w_1 = 6 (B0 B2)^2,       w_2 = 3 (B0 B1)^2
//   side = sum w_k q_k / sum w_k,  q_k = c + t_k/12 + sigma_k s_k/4
// (t, s the second / first differences of the reference's beta_k and candidate polynomials,
// SingleGPU/Burgers3d_WENO5/kernels.cu:92-192). side_rev returns d side / d(a..e) times ybar.
template <class T>
void side_rev(bool Z, T a, T b, T c, T d, T e, T ybar, T g[5]) {
  const T t0 = a - 2 * b + c, t1 = b - 2 * c + d, t2 = c - 2 * d + e;
  const T s0 = a - 4 * b + 3 * c, s1 = b - d, s2 = 3 * c - 4 * d + e;
  const T K = T(13) / T(3), E = T(4e-6);
  const T B0 = K * t0 * t0 + s0 * s0 + E, B1 = K * t1 * t1 + s1 * s1 + E, B2 = K * t2 * t2 + s2 * s2 + E;
  const T q0 = c + t0 / 12 + s0 / 4, q1 = c + t1 / 12 - s1 / 4, q2 = c + t2 / 12 - s2 / 4;
  T w0, w1, w2, tau = 0;
  if (Z) {
    tau = std::fabs(B0 - B2);
    w0 = (B0 + tau) * B1 * B2;
    w1 = 6 * (B1 + tau) * B0 * B2;
    w2 = 3 * (B2 + tau) * B0 * B1;
  } else {
    w0 = (B1 * B2) * (B1 * B2);
    w1 = 6 * (B0 * B2) * (B0 * B2);
    w2 = 3 * (B0 * B1) * (B0 * B1);
  }
  const T D = w0 + w1 + w2;
  const T side = (w0 * q0 + w1 * q1 + w2 * q2) / D;
  const T Nb = ybar / D;
  const T wb0 = Nb * (q0 - side), wb1 = Nb * (q1 - side), wb2 = Nb * (q2 - side);
  const T qb0 = Nb * w0, qb1 = Nb * w1, qb2 = Nb * w2;
  T Bb0 = 0, Bb1 = 0, Bb2 = 0;
  if (Z) {
    T taub = wb0 * B1 * B2 + 6 * wb1 * B0 * B2 + 3 * wb2 * B0 * B1;
    Bb0 += wb0 * B1 * B2 + 6 * wb1 * (B1 + tau) * B2 + 3 * wb2 * (B2 + tau) * B1;
    Bb1 += wb0 * (B0 + tau) * B2 + 6 * wb1 * B0 * B2 + 3 * wb2 * (B2 + tau) * B0;
    Bb2 += wb0 * (B0 + tau) * B1 + 6 * wb1 * (B1 + tau) * B0 + 3 * wb2 * B0 * B1;
    const T sg = B0 > B2 ? T(1) : (B0 < B2 ? T(-1) : T(0));
    Bb0 += sg * taub;
    Bb2 -= sg * taub;
  } else {
    const T p12 = B1 * B2, p02 = B0 * B2, p01 = B0 * B1;
    Bb0 += 12 * wb1 * p02 * B2 + 6 * wb2 * p01 * B1;
    Bb1 += 2 * wb0 * p12 * B2 + 6 * wb2 * p01 * B0;
    Bb2 += 2 * wb0 * p12 * B1 + 12 * wb1 * p02 * B0;
  }
  const T tb0 = 2 * K * t0 * Bb0 + qb0 / 12, tb1 = 2 * K * t1 * Bb1 + qb1 / 12, tb2 = 2 * K * t2 * Bb2 + qb2 / 12;
  const T sb0 = 2 * s0 * Bb0 + qb0 / 4, sb1 = 2 * s1 * Bb1 - qb1 / 4, sb2 = 2 * s2 * Bb2 - qb2 / 4;
  const T cb = qb0 + qb1 + qb2;
  g[0] = tb0 + sb0;
  g[1] = -2 * tb0 + tb1 - 4 * sb0 + sb1;
  g[2] = tb0 - 2 * tb1 + tb2 + 3 * sb0 + 3 * sb2 + cb;
  g[3] = tb1 - 2 * tb2 - sb1 - 4 * sb2;
  g[4] = tb2 + sb2;
}

// lam_out = lam + dt * J(v)^T lam for one stage input v (periodic, local LF).
template <class T>
void burgers_stage_adjoint(const BurgersCfg& c, const T* v, const T* lam, T dt, T* out) {
  const int64_t nx = c.nx, ny = c.ny, nz = c.nz;
  const size_t n = (size_t)nx * ny * nz;
  std::vector<T> GP(n, T(0)), GM(n, T(0));
  const int64_t dims[3] = {nx, ny, nz};
  const T rd[3] = {T(1) / (T)c.dx, T(1) / (T)c.dy, T(1) / (T)c.dz};
  auto fp = [](T u) { return u * (u / 4 + std::fabs(u) / 2); };
  auto fm = [](T u) { return u * (u / 4 - std::fabs(u) / 2); };
  for (int ax = 0; ax < 3; ++ax) {
    for (int64_t k = 0; k < nz; ++k)
      for (int64_t j = 0; j < ny; ++j)
        for (int64_t i = 0; i < nx; ++i) {
          int64_t p[3] = {i, j, k};
          auto idx = [&](int64_t off) {
            int64_t q[3] = {p[0], p[1], p[2]};
            q[ax] = ((q[ax] + off) % dims[ax] + dims[ax]) % dims[ax];
            return (size_t)(q[0] + nx * (q[1] + ny * q[2]));
          };
          // face at p + 1/2 along ax
          const T psi = rd[ax] * (lam[idx(1)] - lam[idx(0)]);
          T P[5], M[5];
          side_rev<T>(c.weno_z != 0, fp(v[idx(-2)]), fp(v[idx(-1)]), fp(v[idx(0)]), fp(v[idx(1)]), fp(v[idx(2)]), psi,
                      P);
          side_rev<T>(c.weno_z != 0, fm(v[idx(3)]), fm(v[idx(2)]), fm(v[idx(1)]), fm(v[idx(0)]), fm(v[idx(-1)]),
                      psi, M);
          for (int q = 0; q < 5; ++q) {
            GP[idx(q - 2)] += P[q];
            GM[idx(3 - q)] += M[q];
          }
        }
  }
  for (size_t o = 0; o < n; ++o) {
    const T u = v[o];
    const T jt = (u / 2 + std::fabs(u)) * GP[o] + (u / 2 - std::fabs(u)) * GM[o];
    out[o] = lam[o] + dt * jt;
  }
}

// Adjoint of one SSP-RK3 step from its stage inputs u_n, u1, u2: lam (dJ/du^{n+1}) becomes
// dJ/du^n. Stage s output: a_s u^n + b_s (v + dt L(v)), (a, b) = (0, 1), (3/4, 1/4), (1/3, 2/3).
template <class T>
void burgers_step_adjoint(const BurgersCfg& c, const T* un, const T* u1, const T* u2, T dt, T* lam) {
  const size_t n = (size_t)c.nx * c.ny * c.nz;
  std::vector<T> t(n), l2(n), l1(n), acc(n);
  burgers_stage_adjoint<T>(c, u2, lam, dt, t.data());
  for (size_t o = 0; o < n; ++o) { l2[o] = T(2) / T(3) * t[o]; acc[o] = lam[o] / T(3); }
  burgers_stage_adjoint<T>(c, u1, l2.data(), dt, t.data());
  for (size_t o = 0; o < n; ++o) { l1[o] = T(0.25) * t[o]; acc[o] += T(0.75) * l2[o]; }
  burgers_stage_adjoint<T>(c, un, l1.data(), dt, t.data());
  for (size_t o = 0; o < n; ++o) lam[o] = acc[o] + t[o];
}

// ------------------------------------------------------------------------------------------
// The MATLAB prototypes of the inviscid Burgers solver (Matlab_Prototipes/InviscidBurgersNd),
// restated: the residual functions WENO{5,7}resAdv_{X,Y,Z}.m / WENO{5,7}resAdv1d.m and the
// solver loops of LFWENO{5,7}FDM{1,2,3}d.m. Flux f = u^2/2 (the drivers' 'burgers' case).
//   * Split f+- = (f +- a u)/2 with a = |u| at every node (the X/Y/Z files) or a = max|u| of
//     the line (the 1d files).
//   * Along each axis the line is extended by copies of its end values (2 left / 3 right for
//     WENO5, 3 left / 4 right for WENO7: a clamped index); fluxes are formed at the faces
//     i+1/2, i = 0..N-1, and the face left of cell 0 is taken as 0, so
//     res_i = (F_{i+1/2} - F_{i-1/2}) / h with F_{-1/2} = 0 (WENO7resAdv_X.m:56-58, 148).
//   * WENO5: Jiang-Shu weights d_k / (eps + beta_k)^2 (WENO5resAdv_X.m:62-120).
//   * WENO7: the seven-point WENO of Balsara & Shu (J. Comput. Phys. 160 (2000) 405-452):
//     four cubic candidates with linear weights 1/35, 12/35, 18/35, 4/35 and weights
//     d_k / (eps + beta_k)^2, eps = 1e-6; the smoothness indicators are the prototype's
//     integer quadratic forms (WENO7resAdv_X.m:75-82).
//   * Both are evaluated in the prototypes' operand order: the FP64 results equal theirs bit
//     for bit (WENO7's indicators cancel to rounding residues that are not small against eps,
//     so another summation order would differ by far more than one rounding).
//   * Time loops: dt = CFL dx / max|u| trimmed to land on tEnd; WENO5 with SSP-RK3, WENO7 with
//     the five-stage, fourth-order low-storage Runge-Kutta scheme of Carpenter & Kennedy
//     (NASA TM-109112, 1994) in its 2N-storage form r = A_s r + dt R(u), u = u - B_s r
//     (LFWENO7FDM3d.m:65-104).
// ------------------------------------------------------------------------------------------
namespace {

// The face fluxes below are evaluated in the prototypes' own operand order (sums left to right
// as the .m files write them, `a - k*b` as `a + (-k)*b`, which rounds identically), so the FP64
// results are bit for bit those of the prototypes. Every smoothness indicator of WENO7 has the
// form  x2*(k0*x2 + k1*x3) + x0*(((k2*xb + k3*xc) + k4*xd) + k5*x3) + k6*x3*x3
//        + x1*((k7*xs + k8*xt) + k9*x3)  over its four cells x0..x3 (WENO7resAdv_X.m:75-82).
struct W7Beta {
  int b, c, d;      // cells of the second term's first three products
  int s, t;         // cells of the fourth term's first two products
  double k[10];
};
constexpr W7Beta kW7Beta[4] = {
    {2, 1, 0, 2, 1, {134241, -114894, 56694, -47214, 6649, -22778, 25729, -210282, 85641, 86214}},
    {1, 0, 2, 1, 2, {41001, -30414, -19374, 3169, 19014, -5978, 6649, 33441, -70602, 23094}},
    {0, 1, 2, 1, 2, {33441, -19374, 6649, -30414, 23094, -5978, 3169, 41001, -70602, 19014}},
    {0, 1, 2, 1, 2, {85641, -47214, 25729, -114894, 86214, -22778, 6649, 134241, -210282, 56694}},
};
// Candidate reconstructions (c0 x0 + c1 x1 + c2 x2 + c3 x3)/12 of the two split parts: rows for
// the part moving towards +x (cells i-3+k .. i+k) and towards -x (cells i-2+k .. i+1+k).
constexpr double kW7PolyPlus[4][4] = {{-3, 13, -23, 25}, {1, -5, 13, 3}, {-1, 7, 7, -1}, {3, 13, -5, 1}};
constexpr double kW7PolyMinus[4][4] = {{1, -5, 13, 3}, {-1, 7, 7, -1}, {3, 13, -5, 1}, {25, -23, 13, -3}};
constexpr double kW7LinPlus[4] = {1. / 35., 12. / 35., 18. / 35., 4. / 35.};
constexpr double kW7LinMinus[4] = {4. / 35., 18. / 35., 12. / 35., 1. / 35.};

// One split part's WENO7 face value from its seven cells f[0..6] (its four stencils are
// f[k..k+3]); `poly` and `lin` select the +x or -x part.
template <class T>
inline T weno7_part(const T f[7], const double (&poly)[4][4], const double (&lin)[4]) {
  const T eps = (T)1e-6;
  T a[4];
  for (int k = 0; k < 4; ++k) {
    const T* x = f + k;
    const W7Beta& B = kW7Beta[k];
    const double* q = B.k;
    const T t1 = x[2] * ((T)q[0] * x[2] + (T)q[1] * x[3]);
    const T t2 = x[0] * ((((T)q[2] * x[B.b] + (T)q[3] * x[B.c]) + (T)q[4] * x[B.d]) + (T)q[5] * x[3]);
    const T t3 = (T)q[6] * (x[3] * x[3]);
    const T t4 = x[1] * (((T)q[7] * x[B.s] + (T)q[8] * x[B.t]) + (T)q[9] * x[3]);
    const T beta = ((t1 + t2) + t3) + t4;
    a[k] = (T)lin[k] / ((eps + beta) * (eps + beta));
  }
  const T sum = ((a[0] + a[1]) + a[2]) + a[3];
  T h = 0;
  for (int k = 0; k < 4; ++k) {
    const T* x = f + k;
    const T cand = (((T)poly[k][0] * x[0] + (T)poly[k][1] * x[1]) + (T)poly[k][2] * x[2]) + (T)poly[k][3] * x[3];
    const T term = (a[k] / sum) * cand / (T)12;
    h = k == 0 ? term : h + term;
  }
  return h;
}

// WENO7 reconstruction at the face between f[3] and f[4] of the part moving towards +x, from the
// seven cells f[0..6] around it (the prototypes' hn).
template <class T>
inline T weno7_side(const T f[7]) {
  return weno7_part<T>(f, kW7PolyPlus, kW7LinPlus);
}

// One split part's WENO5 face value in WENO5resAdv_X.m's order (:62-120): cells x[0..4], linear
// weights d, candidates (c . x[k..k+2]) / 6 with rows `poly`.
template <class T>
inline T weno5_part(const T x[5], const double (&d)[3], const double (&poly)[3][3]) {
  const T eps = (T)1e-6, c1312 = (T)(13. / 12.), c14 = (T)(1. / 4.);
  // (a, b) of 13/12 a^2 + 1/4 b^2 per stencil
  const T a0 = (x[0] - (T)2 * x[1]) + x[2], b0 = (x[0] - (T)4 * x[1]) + (T)3 * x[2];
  const T a1 = (x[1] - (T)2 * x[2]) + x[3], b1 = x[1] - x[3];
  const T a2 = (x[2] - (T)2 * x[3]) + x[4], b2 = ((T)3 * x[2] - (T)4 * x[3]) + x[4];
  const T B[3] = {c1312 * (a0 * a0) + c14 * (b0 * b0), c1312 * (a1 * a1) + c14 * (b1 * b1),
                  c1312 * (a2 * a2) + c14 * (b2 * b2)};
  T al[3];
  for (int k = 0; k < 3; ++k) al[k] = (T)d[k] / ((eps + B[k]) * (eps + B[k]));
  const T sum = (al[0] + al[1]) + al[2];
  T h = 0;
  for (int k = 0; k < 3; ++k) {
    const T cand = ((T)poly[k][0] * x[k] + (T)poly[k][1] * x[k + 1]) + (T)poly[k][2] * x[k + 2];
    const T term = (al[k] / sum) * cand / (T)6;
    h = k == 0 ? term : h + term;
  }
  return h;
}
constexpr double kW5LinPlus[3] = {1. / 10., 6. / 10., 3. / 10.};
constexpr double kW5LinMinus[3] = {3. / 10., 6. / 10., 1. / 10.};
constexpr double kW5PolyPlus[3][3] = {{2, -7, 11}, {-1, 5, 2}, {2, 5, -1}};
constexpr double kW5PolyMinus[3][3] = {{-1, 5, 2}, {2, 5, -1}, {11, -7, 2}};

// The two split parts' face values (hp, hn) at i+1/2: `part(j, side)` gives cell i+j of the
// part moving towards +x (side 0) or -x (side 1).
template <class T, class G>
inline void proto_face(int order, G part, T* hp, T* hn) {
  if (order == 7) {
    T p[7], m[7];
    for (int j = 0; j < 7; ++j) {
      p[j] = part(j - 3, 0);  // cells i-3 .. i+3
      m[j] = part(j - 2, 1);  // cells i-2 .. i+4
    }
    *hn = weno7_part<T>(p, kW7PolyPlus, kW7LinPlus);
    *hp = weno7_part<T>(m, kW7PolyMinus, kW7LinMinus);
    return;
  }
  T p[5], m[5];
  for (int j = 0; j < 5; ++j) {
    p[j] = part(j - 2, 0);  // cells i-2 .. i+2
    m[j] = part(j - 1, 1);  // cells i-1 .. i+3
  }
  *hn = weno5_part<T>(p, kW5LinPlus, kW5PolyPlus);
  *hp = weno5_part<T>(m, kW5LinMinus, kW5PolyMinus);
}

// res = d f(u) / d axis on every node, by the prototype residual function of `order` (5 or 7);
// line_max = 1 takes a = max|u| along each line (the 1d files), else a = |u| per node.
template <class T>
void proto_residual(int order, int axis, int line_max, int nx, int ny, int nz, double h, const T* u, T* res) {
  const int n[3] = {nx, ny, nz};
  const int N = n[axis];
  const size_t stride = axis == 0 ? 1 : axis == 1 ? (size_t)nx : (size_t)nx * ny;
  const int o1 = axis == 0 ? 1 : 0, o2 = axis == 2 ? 1 : 2;  // the two other axes
  const int lines = n[o1] * n[o2];
#pragma omp parallel for schedule(static)
  for (int l = 0; l < lines; ++l) {
    int c[3] = {0, 0, 0};
    c[o1] = l % n[o1];
    c[o2] = l / n[o1];
    const T* line = u + (size_t)c[0] + (size_t)nx * ((size_t)c[1] + (size_t)ny * c[2]);
    T* out = res + (line - u);
    std::vector<T> fp(N), fm(N);
    T amax = 0;
    if (line_max)
      for (int i = 0; i < N; ++i) amax = std::max(amax, (T)std::fabs(line[(size_t)i * stride]));
    for (int i = 0; i < N; ++i) {
      const T v = line[(size_t)i * stride];
      const T f = v * v / (T)2;
      const T a = line_max ? amax : (T)std::fabs(v);
      fp[i] = (T)0.5 * (f + a * v);
      fm[i] = (T)0.5 * (f - a * v);
    }
    T hp0 = 0, hn0 = 0;  // the face left of cell 0 is zero
    for (int i = 0; i < N; ++i) {
      auto part = [&](int j, int side) -> T {
        const int k = std::min(std::max(i + j, 0), N - 1);
        return side == 0 ? fp[k] : fm[k];
      };
      T hp1, hn1;
      proto_face<T>(order, part, &hp1, &hn1);
      out[(size_t)i * stride] = (((hp1 + hn1) - hp0) - hn0) / (T)h;  // res = (hp+hn-hp'-hn')/dx
      hp0 = hp1;
      hn0 = hn1;
    }
  }
}

// Carpenter & Kennedy's five-stage fourth-order 2N-storage Runge-Kutta coefficients (the
// published rational values, also those of LFWENO7FDM3d.m:66-79).
constexpr double kLsrkA[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                              -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
constexpr double kLsrkB[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                              1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                              2277821191437.0 / 14882151754819.0};

// Sum of the residuals of every axis of an ndim-dimensional grid, accumulated in axis order.
template <class T>
void proto_rhs(int order, int ndim, int nx, int ny, int nz, const double h[3], const T* u, T* acc, T* tmp) {
  const size_t n = (size_t)nx * ny * nz;
  proto_residual<T>(order, 0, ndim == 1, nx, ny, nz, h[0], u, acc);
  for (int ax = 1; ax < ndim; ++ax) {
    proto_residual<T>(order, ax, 0, nx, ny, nz, h[ax], u, tmp);
    for (size_t o = 0; o < n; ++o) acc[o] += tmp[o];
  }
}

// The prototype solver loop; returns the number of time steps, the end time in *t_out.
template <class T>
int64_t proto_run(int order, int ndim, int nx, int ny, int nz, const double h[3], double cfl, double tEnd,
                  int64_t max_steps, T* u, double* t_out) {
  const size_t n = (size_t)nx * ny * nz;
  std::vector<T> L(n), tmp(n), uo(n), r(n, (T)0);
  double t = 0;
  int64_t it = 0;
  while (t < tEnd && it < max_steps) {
    T umax = 0;
    for (size_t o = 0; o < n; ++o) umax = std::max(umax, (T)std::fabs(u[o]));
    double dt = cfl * h[0] / (double)umax;
    if (t + dt > tEnd) dt = tEnd - t;
    t += dt;
    ++it;
    const T tdt = (T)dt;
    if (order == 7) {
      for (int s = 0; s < 5; ++s) {
        proto_rhs<T>(order, ndim, nx, ny, nz, h, u, L.data(), tmp.data());
        for (size_t o = 0; o < n; ++o) {
          r[o] = (T)kLsrkA[s] * r[o] + tdt * L[o];
          u[o] = u[o] - (T)kLsrkB[s] * r[o];
        }
      }
    } else {
      std::memcpy(uo.data(), u, n * sizeof(T));
      proto_rhs<T>(order, ndim, nx, ny, nz, h, u, L.data(), tmp.data());
      for (size_t o = 0; o < n; ++o) u[o] = uo[o] - tdt * L[o];
      proto_rhs<T>(order, ndim, nx, ny, nz, h, u, L.data(), tmp.data());
      for (size_t o = 0; o < n; ++o) u[o] = (T)0.75 * uo[o] + (T)0.25 * (u[o] - tdt * L[o]);
      proto_rhs<T>(order, ndim, nx, ny, nz, h, u, L.data(), tmp.data());
      for (size_t o = 0; o < n; ++o) u[o] = (uo[o] + (T)2 * (u[o] - tdt * L[o])) / (T)3;
    }
  }
  *t_out = t;
  return it;
}

}  // namespace

extern "C" {

// ----------------------------------------------------------------------------- RNG
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  philox4x32_10(ctr, key, out);
}
void orc_philox_u01x2(uint32_t seed, uint32_t stream, uint64_t idx, double* a, double* b) {
  philox_u01x2(seed, stream, idx, a, b);
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// ----------------------------------------------------------------------------- heat
#define HEAT_CFG                                                                             \
  HeatCfg c{ndim, nx, ny, nz, order, frozen, zero_boundary, periodic, kx, ky, kz, dt};

void orc_heat_stage_f64(int ndim, int nx, int ny, int nz, int order, int frozen, int zero_boundary,
                        int periodic, double kx, double ky, double kz, double dt, int stage,
                        const double* uin, const double* un, double* out) {
  HEAT_CFG heat_stage<double>(c, stage, uin, un, out);
}
void orc_heat_stage_f32(int ndim, int nx, int ny, int nz, int order, int frozen, int zero_boundary,
                        int periodic, double kx, double ky, double kz, double dt, int stage,
                        const float* uin, const float* un, float* out) {
  HEAT_CFG heat_stage<float>(c, stage, uin, un, out);
}
void orc_heat_run_f64(int ndim, int nx, int ny, int nz, int order, int frozen, int zero_boundary,
                      int periodic, double kx, double ky, double kz, double dt, int time,
                      int64_t nsteps, double* u) {
  HEAT_CFG heat_run<double>(c, time, nsteps, u);
}
void orc_heat_run_f32(int ndim, int nx, int ny, int nz, int order, int frozen, int zero_boundary,
                      int periodic, double kx, double ky, double kz, double dt, int time,
                      int64_t nsteps, float* u) {
  HEAT_CFG heat_run<float>(c, time, nsteps, u);
}

void orc_heat_stage_f32_fma(int ndim, int nx, int ny, int nz, int order, int frozen, int zero_boundary,
                            int periodic, double kx, double ky, double kz, double dt, int stage,
                            const float* uin, const float* un, float* out) {
  HEAT_CFG heat_stage_fma<float>(c, stage, uin, un, out);
}
void orc_heat_run_f32_fma(int ndim, int nx, int ny, int nz, int order, int frozen, int zero_boundary,
                          int periodic, double kx, double ky, double kz, double dt, int time,
                          int64_t nsteps, float* u) {
  HEAT_CFG heat_run_fma<float>(c, time, nsteps, u);
}
void orc_heat_stage_f64_fma(int ndim, int nx, int ny, int nz, int order, int frozen, int zero_boundary,
                            int periodic, double kx, double ky, double kz, double dt, int stage,
                            const double* uin, const double* un, double* out) {
  HEAT_CFG heat_stage_fma<double>(c, stage, uin, un, out);
}
void orc_heat_run_f64_fma(int ndim, int nx, int ny, int nz, int order, int frozen, int zero_boundary,
                          int periodic, double kx, double ky, double kz, double dt, int time,
                          int64_t nsteps, double* u) {
  HEAT_CFG heat_run_fma<double>(c, time, nsteps, u);
}

// Reference heat dt and final time (SingleGPU/Diffusion3d_baselineCode/main.cpp:55-63,
// SingleGPU/Diffusion2d/main.cpp:52-58). L/W/H are integers there (parsed with atoi).
void orc_heat_ref_constants(int ndim, double C, int L, int W, int H, int nx, int ny, int nz,
                            int iters, double* dx, double* dy, double* dz, double* dt,
                            double* k_x, double* k_y, double* k_z, double* tFinal) {
  *dx = (double)L / (nx - 1);
  *dy = (double)W / (ny - 1);
  *dz = (ndim == 3) ? (double)H / (nz - 1) : 0.0;
  if (ndim == 3)
    *dt = 1 / (2 * C * (1 / *dx / *dx + 1 / *dy / *dy + 1 / *dz / *dz)) * 0.9;
  else
    *dt = 1 / (2 * C * (1 / *dx / *dx + 1 / *dy / *dy)) * 0.9;
  *k_x = C / (12 * *dx * *dx);
  *k_y = C / (12 * *dy * *dy);
  *k_z = (ndim == 3) ? C / (12 * *dz * *dz) : 0.0;
  *tFinal = 0.1 + *dt * iters;
}

// Reference heat initial condition 3 (SingleGPU/Diffusion3d_baselineCode/tools.cpp:128-139 with
// EXP_DISTRIBUTION of acoustics3d.h:29; 2D: SingleGPU/Diffusion2d/tools.cpp:109-119).
void orc_ic_heat_ref(int ndim, int nx, int ny, int nz, double dx, double dy, double dz, double* u) {
  const int NZ = ndim == 3 ? nz : 1;
  for (int k = 0; k < NZ; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t o = (size_t)i + (size_t)nx * j + (size_t)nx * ny * k;
        double r2 = (-5 + i * dx) * (-5 + i * dx) + (-5 + j * dy) * (-5 + j * dy);
        if (ndim == 3) r2 += (-5 + k * dz) * (-5 + k * dz);
        u[o] = std::exp(-(r2) / (4 * 1.0 * 0.1));
        bool face = i == 0 || i == nx - 1 || j == 0 || j == ny - 1;
        if (ndim == 3) face = face || k == 0 || k == nz - 1;
        if (face) u[o] = 0.0;
      }
}

// MATLAB accuracy study, literal: Matlab_Prototipes/DiffusionNd/diffusion{1,2,3}dTest.m with
// Laplace{1,2,3}d.m ("OMP" index range in 3D, Laplace3d.m:38-53). O4 + SSP-RK3, outermost layer
// reset to 0 after each step, dt trimmed AFTER the step and t advanced by the trimmed dt
// (diffusion3dTest.m:55-68). Returns the number of steps; L1/L2/Linf as the .m files print them.
int orc_heat_accuracy(int dim, int nc, double tFinal, double param, double* L1, double* L2,
                      double* Linf) {
  const double D = 1.0, t0 = 0.1, L = 10.0;
  const double dx = L / (nc - 1);
  const double Dx = D / (dx * dx);
  const int nx = nc, ny = dim >= 2 ? nc : 1, nz = dim == 3 ? nc : 1;
  const size_t n = (size_t)nx * ny * nz;
  std::vector<double> u(n), uo(n), dF(n), uE(n);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double x = -L / 2 + i * dx, y = -L / 2 + j * dx, z = -L / 2 + k * dx;
        double r2 = x * x;
        if (dim >= 2) r2 += y * y;
        if (dim == 3) r2 += z * z;
        size_t o = (size_t)i + (size_t)nx * j + (size_t)nx * ny * k;
        u[o] = std::exp(-r2 / (4 * 1.0 * t0));
        double amp = dim == 1 ? std::sqrt(t0 / tFinal) : dim == 2 ? t0 / tFinal : std::pow(t0 / tFinal, 1.5);
        uE[o] = amp * std::exp(-r2 / (4 * 1.0 * tFinal));
      }
  double dt;
  if (dim == 1) dt = 1 / (2 * D * (1 / (dx * dx))) * param;
  else if (dim == 2) dt = 1 / (2 * D * (1 / (dx * dx) + 1 / (dx * dx))) * param;
  else dt = 1 / (2 * D * (1 / (dx * dx) + 1 / (dx * dx) + 1 / (dx * dx))) * param;

  auto lap = [&](const std::vector<double>& w) {
    std::fill(dF.begin(), dF.end(), 0.0);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          bool in = i >= 2 && i <= nx - 3;
          if (dim >= 2) in = in && j >= 2 && j <= ny - 3;
          if (dim == 3) in = in && k >= 2 && k <= nz - 3;
          if (!in) continue;
          size_t o = (size_t)i + (size_t)nx * j + (size_t)nx * ny * k;
          size_t sy = nx, sz = (size_t)nx * ny;
          double v;
          if (dim < 3) {  // Laplace{1,2}d.m: each axis from its + side (i+2 first)
            v = Dx / 12 * (-w[o + 2] + 16 * w[o + 1] - 30 * w[o] + 16 * w[o - 1] - w[o - 2]);
            if (dim == 2) v = v + Dx / 12 * (-w[o + 2 * sy] + 16 * w[o + sy] - 30 * w[o] + 16 * w[o - sy] - w[o - 2 * sy]);
          } else {  // Laplace3d.m's "OMP" branch (:29-52): each axis from its - side (o-2 first)
            v = Dx / 12 * (-w[o - 2] + 16 * w[o - 1] - 30 * w[o] + 16 * w[o + 1] - w[o + 2]) +
                Dx / 12 * (-w[o - 2 * sy] + 16 * w[o - sy] - 30 * w[o] + 16 * w[o + sy] - w[o + 2 * sy]);
            v = v + Dx / 12 * (-w[o - 2 * sz] + 16 * w[o - sz] - 30 * w[o] + 16 * w[o + sz] - w[o + 2 * sz]);
          }
          dF[o] = v;
        }
  };
  double t = t0;
  int it = 0;
  while (t < tFinal) {
    uo = u;
    lap(u);
    for (size_t o = 0; o < n; ++o) u[o] = uo[o] + dt * dF[o];
    lap(u);
    for (size_t o = 0; o < n; ++o) u[o] = 0.75 * uo[o] + 0.25 * (u[o] + dt * dF[o]);
    lap(u);
    for (size_t o = 0; o < n; ++o) u[o] = (uo[o] + 2 * (u[o] + dt * dF[o])) / 3;
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          bool b = i == 0 || i == nx - 1;
          if (dim >= 2) b = b || j == 0 || j == ny - 1;
          if (dim == 3) b = b || k == 0 || k == nz - 1;
          if (b) u[(size_t)i + (size_t)nx * j + (size_t)nx * ny * k] = 0.0;
        }
    if (t + dt > tFinal) dt = tFinal - t;
    it = it + 1;
    t = t + dt;
  }
  const double vol = dim == 1 ? dx : dim == 2 ? dx * dx : dx * dx * dx;
  double s1 = 0, s2 = 0, mx = 0;
  for (size_t o = 0; o < n; ++o) {
    double e = std::fabs(uE[o] - u[o]);
    s1 += e;
    s2 += e * e;
    mx = std::max(mx, e);
  }
  *L1 = vol * s1;
  *L2 = std::sqrt(vol * s2);
  *Linf = mx;
  return it;
}

// Seeded configuration initial conditions (all draws from Philox4x32-10).
// 2D: exp(-((x-.5)^2+(y-.5)^2)/0.01) + N(0, sigma^2) on nodes x_i = i/(n-1); boundary = 0.
// Noise draw for node o uses stream 1, index o (Box-Muller on the two uniforms).
void orc_ic_heat2d_gauss_noise(int nx, int ny, uint32_t seed, double sigma, double* u) {
  const double hx = 1.0 / (nx - 1), hy = 1.0 / (ny - 1);
  const double two_pi = 6.283185307179586476925286766559;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      size_t o = (size_t)i + (size_t)nx * j;
      double x = i * hx, y = j * hy;
      double g = std::exp(-((x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5)) / 0.01);
      double a, b;
      philox_u01x2(seed, 1u, (uint64_t)o, &a, &b);
      double z = std::sqrt(-2.0 * std::log(1.0 - a)) * std::cos(two_pi * b);
      u[o] = g + sigma * z;
      if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1) u[o] = 0.0;
    }
}

// Blob parameters: blob m uses stream 2, draws 2m and 2m+1 -> (cx, cy), (cz, sigma).
void orc_heat3d_blob_params(uint32_t seed, int nblobs, double* params /* 4*nblobs */) {
  for (int m = 0; m < nblobs; ++m) {
    double a, b, c, d;
    philox_u01x2(seed, 2u, (uint64_t)(2 * m), &a, &b);
    philox_u01x2(seed, 2u, (uint64_t)(2 * m + 1), &c, &d);
    params[4 * m + 0] = 0.2 + 0.6 * a;
    params[4 * m + 1] = 0.2 + 0.6 * b;
    params[4 * m + 2] = 0.2 + 0.6 * c;
    params[4 * m + 3] = 0.02 + 0.06 * d;
  }
}

// 3D: sum of blobs exp(-|x-c|^2/(2 sigma^2)) on nodes x_i = i/(n-1) of [0,1]^3; boundary = 0.
void orc_ic_heat3d_blobs(int nx, int ny, int nz, uint32_t seed, int nblobs, double* u) {
  std::vector<double> p(4 * (size_t)nblobs);
  orc_heat3d_blob_params(seed, nblobs, p.data());
  const double hx = 1.0 / (nx - 1), hy = 1.0 / (ny - 1), hz = 1.0 / (nz - 1);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t o = (size_t)i + (size_t)nx * j + (size_t)nx * ny * k;
        double x = i * hx, y = j * hy, z = k * hz, s = 0.0;
        for (int m = 0; m < nblobs; ++m) {
          double ddx = x - p[4 * m], ddy = y - p[4 * m + 1], ddz = z - p[4 * m + 2], sg = p[4 * m + 3];
          s += std::exp(-(ddx * ddx + ddy * ddy + ddz * ddz) / (2 * sg * sg));
        }
        bool face = i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k == nz - 1;
        u[o] = face ? 0.0 : s;
      }
}

// Fourier-mode parameters: mode m draws (stream 3) wave vectors n in [-4,4]^3 \ {0} with
// |n| <= 4 by rejection (draw index advanced per attempt), then amplitude a ~ U[0, amax]
// and phase ~ U[0, 2 pi) from stream 4, index m. params = (n1, n2, n3, a, phi) per mode.
void orc_burgers_fourier_params(uint32_t seed, int nmodes, double amax, double* params) {
  const double two_pi = 6.283185307179586476925286766559;
  uint64_t idx = 0;
  for (int m = 0; m < nmodes; ++m) {
    int n1, n2, n3;
    for (;;) {
      double a, b, c, d;
      philox_u01x2(seed, 3u, idx++, &a, &b);
      philox_u01x2(seed, 3u, idx++, &c, &d);
      n1 = (int)std::floor(a * 9.0) - 4;
      n2 = (int)std::floor(b * 9.0) - 4;
      n3 = (int)std::floor(c * 9.0) - 4;
      int r2 = n1 * n1 + n2 * n2 + n3 * n3;
      if (r2 > 0 && r2 <= 16) break;
    }
    double a, b;
    philox_u01x2(seed, 4u, (uint64_t)m, &a, &b);
    params[5 * m + 0] = n1;
    params[5 * m + 1] = n2;
    params[5 * m + 2] = n3;
    params[5 * m + 3] = amax * a;
    params[5 * m + 4] = two_pi * b;
  }
}

// u0 = 0.5 + sum_m a_m cos(pi n_m . x + phi_m) on the periodic cell centres
// x_i = (i + 1/2) L/N of [0, L)^3 (L = 2).
void orc_ic_burgers_fourier(int nx, int ny, int nz, double L, uint32_t seed, int nmodes,
                            double amax, double* u) {
  std::vector<double> p(5 * (size_t)nmodes);
  orc_burgers_fourier_params(seed, nmodes, amax, p.data());
  const double pi = 3.14159265358979323846264338327950288;
  const double hx = L / nx, hy = L / ny, hz = L / nz;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double x = (i + 0.5) * hx, y = (j + 0.5) * hy, z = (k + 0.5) * hz, s = 0.5;
        for (int m = 0; m < nmodes; ++m)
          s += p[5 * m + 3] * std::cos(pi * (p[5 * m] * x + p[5 * m + 1] * y + p[5 * m + 2] * z) + p[5 * m + 4]);
        u[(size_t)i + (size_t)nx * j + (size_t)nx * ny * k] = s;
      }
}

// Reference Burgers initial condition 3 (SingleGPU/Burgers3d_WENO5/tools.cpp:126-137,
// GAUSSIAN_DISTRIBUTION of Burgers.h:41) at nodes (i dx, j dy, k dz).
void orc_ic_burgers_ref(int nx, int ny, int nz, double dx, double dy, double dz, double* u) {
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double x = i * dx, y = j * dy, z = k * dz;
        u[(size_t)i + (size_t)nx * j + (size_t)nx * ny * k] =
            1.0 * std::exp(-((x - 1.0) * (x - 1.0) + (y - 1.0) * (y - 1.0) + (z - 1.0) * (z - 1.0)) / 0.1);
      }
}

// ----------------------------------------------------------------------------- Burgers
#define BURG_CFG                                                                               \
  BurgersCfg c{nx, ny, nz, weno_z, lf_global, periodic, bug_b2, dx, dy, dz, kx, ky, kz};
#define BURG_ARGS                                                                              \
  int nx, int ny, int nz, int weno_z, int lf_global, int periodic, int bug_b2, double dx,      \
      double dy, double dz, double kx, double ky, double kz

void orc_burgers_rhs_f64(BURG_ARGS, const double* u, double a_glob, double* Lu) {
  BURG_CFG burgers_rhs<double, double>(c, u, a_glob, Lu);
}
// FP32 state with `div64` selecting FP64 (1) or FP32 (0) weight divisions.
void orc_burgers_rhs_f32(BURG_ARGS, int div64, const float* u, float a_glob, float* Lu) {
  BURG_CFG if (div64) burgers_rhs<float, double>(c, u, a_glob, Lu);
  else burgers_rhs<float, float>(c, u, a_glob, Lu);
}
void orc_burgers_stage_f64(BURG_ARGS, int stage, const double* uin, const double* un, double dt,
                           double* out, double* Lu) {
  BURG_CFG burgers_stage<double, double>(c, stage, uin, un, dt, out, Lu);
}
void orc_burgers_stage_f32(BURG_ARGS, int div64, int stage, const float* uin, const float* un,
                           double dt, float* out, float* Lu) {
  BURG_CFG if (div64) burgers_stage<float, double>(c, stage, uin, un, dt, out, Lu);
  else burgers_stage<float, float>(c, stage, uin, un, dt, out, Lu);
}
int64_t orc_burgers_run_f64(BURG_ARGS, double* u, double tEnd, double CFL, int dt_rule, double C,
                            int64_t max_steps, double* t_out) {
  BURG_CFG return burgers_run<double, double>(c, u, tEnd, CFL, dt_rule, C, max_steps, t_out);
}
int64_t orc_burgers_run_f32(BURG_ARGS, int div64, float* u, double tEnd, double CFL, int dt_rule,
                            double C, int64_t max_steps, double* t_out) {
  BURG_CFG if (div64) return burgers_run<float, double>(c, u, tEnd, CFL, dt_rule, C, max_steps, t_out);
  return burgers_run<float, float>(c, u, tEnd, CFL, dt_rule, C, max_steps, t_out);
}

// The shared-memory program's loop: the baseline loop with its weight normalisation (the interior
// update depends on no node past the grid, so the zero fill plays no part there).
int64_t orc_burgers_run_recip_f64(BURG_ARGS, double* u, double tEnd, double CFL, int dt_rule, double C,
                                  int64_t max_steps, double* t_out) {
  BURG_CFG c.recip = 1;
  return burgers_run<double, double>(c, u, tEnd, CFL, dt_rule, C, max_steps, t_out);
}
void orc_burgers_sweep_all_f64(int axis, int weno_z, int nx, int ny, int nz, double h, const double* u, double* Lu) {
  sweep_all<double>(axis, weno_z, nx, ny, nz, h, u, Lu);
}
void orc_burgers_sweep_all_f32(int axis, int weno_z, int nx, int ny, int nz, double h, const float* u, float* Lu) {
  sweep_all<float>(axis, weno_z, nx, ny, nz, (float)h, u, Lu);
}
void orc_heat_blocking_run_f64(int nx, int ny, int nz, double kx, double ky, double kz, double dt, int64_t iters,
                               double* u) {
  heat_blocking_run<double>(nx, ny, nz, kx, ky, kz, dt, iters, u);
}

// Reference Burgers dt loop alone (no field update): number of steps and final t
// (SingleGPU/Burgers3d_WENO5/main.cpp:127-136).
int64_t orc_burgers_ref_steps(double tEnd, double CFL, double L, double W, double H, int nx, int ny,
                              int nz, double C, double* t_out) {
  double dx = L / (nx - 1), dy = W / (ny - 1), dz = H / (nz - 1);
  double t = 0, dt;
  int64_t it = 0;
  while (t < tEnd) {
    double dt1 = CFL * dx / 1.0;
    double dt2 = 1. / (2 * C * (1 / dx / dx + 1 / dy / dy + 1 / dz / dz)) * 0.9;
    dt = dt1 < dt2 ? dt1 : dt2;
    if ((t + dt) > tEnd) dt = tEnd - t;
    t += dt;
    it += 1;
  }
  *t_out = t;
  return it;
}

double orc_max_abs_f64(const double* u, int64_t n) { return max_abs<double>(u, (size_t)n); }
float orc_max_abs_f32(const float* u, int64_t n) { return max_abs<float>(u, (size_t)n); }


// heat with k(x): one step and the adjoint of one step
void orc_heatk_step_f64(int nx, int ny, int nz, int zb, double cx, double cy, double cz, const double* k,
                        const double* u, double* out) {
  heatk_step<double>(nx, ny, nz, zb, cx, cy, cz, k, u, out);
}
void orc_heatk_step_f32(int nx, int ny, int nz, int zb, double cx, double cy, double cz, const float* k,
                        const float* u, float* out) {
  heatk_step<float>(nx, ny, nz, zb, (float)cx, (float)cy, (float)cz, k, u, out);
}
void orc_heatk_adjoint_f64(int nx, int ny, int nz, int zb, double cx, double cy, double cz, const double* k,
                           const double* u, const double* lam, double* out, double* grad) {
  heatk_adjoint<double>(nx, ny, nz, zb, cx, cy, cz, k, u, lam, out, grad);
}
void orc_heatk_adjoint_f32(int nx, int ny, int nz, int zb, double cx, double cy, double cz, const float* k,
                           const float* u, const float* lam, float* out, float* grad) {
  heatk_adjoint<float>(nx, ny, nz, zb, (float)cx, (float)cy, (float)cz, k, u, lam, out, grad);
}


// Burgers adjoint of one SSP-RK3 step (periodic, local LF): lam in/out.
void orc_burgers_step_adjoint_f64(BURG_ARGS, const double* un, const double* u1, const double* u2, double dt,
                                  double* lam) {
  BURG_CFG burgers_step_adjoint<double>(c, un, u1, u2, dt, lam);
}
void orc_burgers_step_adjoint_f32(BURG_ARGS, const float* un, const float* u1, const float* u2, double dt,
                                  float* lam) {
  BURG_CFG burgers_step_adjoint<float>(c, un, u1, u2, (float)dt, lam);
}

// ------------------------------------------------------------- MATLAB Burgers prototypes
// order 5 or 7; axis 0/1/2 = x/y/z of an x-fastest nx*ny*nz array; line_max 1 = the 1d files.
void orc_proto_residual_f64(int order, int axis, int line_max, int nx, int ny, int nz, double h, const double* u,
                            double* res) {
  proto_residual<double>(order, axis, line_max, nx, ny, nz, h, u, res);
}
// LFWENO{5,7}FDM{ndim}d.m solver loop on u (in place); h = {dx, dy, dz}.
int64_t orc_proto_run_f64(int order, int ndim, int nx, int ny, int nz, const double* h, double cfl, double tEnd,
                          int64_t max_steps, double* u, double* t_out) {
  return proto_run<double>(order, ndim, nx, ny, nz, h, cfl, tEnd, max_steps, u, t_out);
}
// The WENO7 reconstruction of one face from seven cell values (parts moving towards +x).
double orc_weno7_side_f64(const double* f) { return weno7_side<double>(f); }
// Amplification factor R(z) of one Carpenter-Kennedy LSRK(5,4) step on du/dt = z u (dt = 1).
void orc_lsrk54_gain(double zr, double zi, double* gr, double* gi) {
  double ur = 1, ui = 0, rr = 0, ri = 0;
  for (int s = 0; s < 5; ++s) {
    const double lr = zr * ur - zi * ui, li = zr * ui + zi * ur;  // R(u) = -z u, du/dt = -R
    rr = kLsrkA[s] * rr - lr;
    ri = kLsrkA[s] * ri - li;
    ur = ur - kLsrkB[s] * rr;
    ui = ui - kLsrkB[s] * ri;
  }
  *gr = ur;
  *gi = ui;
}

}  // extern "C"
