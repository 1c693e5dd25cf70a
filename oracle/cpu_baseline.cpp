// cpu_baseline.cpp -- the CPU baseline of the heat benchmark: TEST AND MEASUREMENT INFRASTRUCTURE.
//
// The reference has no CPU implementation of its heat path (its loop runs only on the GPU:
// SingleGPU/Diffusion3d_baselineCode/main.cpp:106-122 around kernels.cu:37-64 and :104-142), so
// the CPU figure the benchmark reports beside the GPU one is this restatement of the same update
// loop, written for speed rather than clarity: forward Euler with the O2 7-point (3D) or 5-point
// (2D) Laplacian, the reference's operand order and rounding (built with -ffp-contract=off, so
// its results equal the oracle's heat_run in FP32 bit for bit, x86 and Arm alike), and
//   * two buffers used in turn, no copy per step (one copy at the end when the step count is odd);
//   * an interior loop over x with no boundary test, which the compiler vectorises;
//   * the frozen layers handled by a separate pass over the row ends and the frozen rows/planes;
//   * OpenMP over contiguous (plane, row) ranges, so each thread streams its own planes.
// Only the tests and bench.py's CPU legs call it; the product never does.
#include <omp.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

namespace {

template <class T>
void euler_o2_sweep(int ndim, int64_t nx, int64_t ny, int64_t nz, int F, int zero_boundary, T kx, T ky, T kz, T dt,
                    const T* __restrict u, T* __restrict v) {
  const int64_t sz = nx * ny;
  const bool three = ndim == 3;
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t k = 0; k < nz; ++k)
    for (int64_t j = 0; j < ny; ++j) {
      const int64_t row = k * sz + j * nx;
      const T* __restrict c = u + row;
      T* __restrict o = v + row;
      const bool kfrozen = three && (k < F || k >= nz - F);
      const bool jfrozen = j < F || j >= ny - F;
      const bool outer_row = j == 0 || j == ny - 1 || (three && (k == 0 || k == nz - 1));
      if (kfrozen || jfrozen) {  // a frozen row: copied, or zero on the outermost layer
        if (zero_boundary && outer_row) {
          std::memset(o, 0, sizeof(T) * nx);
        } else {
          std::memcpy(o, c, sizeof(T) * nx);
          if (zero_boundary) o[0] = o[nx - 1] = T(0);  // the row's ends lie on the outermost x layer
        }
        continue;
      }
      for (int64_t i = 0; i < F && i < nx; ++i) o[i] = (zero_boundary && i == 0) ? T(0) : c[i];
      for (int64_t i = std::max<int64_t>(F, nx - F); i < nx; ++i) o[i] = (zero_boundary && i == nx - 1) ? T(0) : c[i];
      const T* __restrict n = c + nx;
      const T* __restrict s = c - nx;
      const int64_t ib = F, ie = nx - F;
      if (three) {
        const T* __restrict t = c + sz;
        const T* __restrict b = c - sz;
#pragma omp simd
        for (int64_t i = ib; i < ie; ++i) {
          const T ce = c[i];
          const T Sx = (c[i + 1] - T(2) * ce) + c[i - 1];
          const T Sy = (n[i] - T(2) * ce) + s[i];
          const T Sz = (t[i] - T(2) * ce) + b[i];
          const T L = (kx * Sx + ky * Sy) + kz * Sz;
          o[i] = ce + dt * L;
        }
      } else {
#pragma omp simd
        for (int64_t i = ib; i < ie; ++i) {
          const T ce = c[i];
          const T Sx = (c[i + 1] - T(2) * ce) + c[i - 1];
          const T Sy = (n[i] - T(2) * ce) + s[i];
          const T L = kx * Sx + ky * Sy;
          o[i] = ce + dt * L;
        }
      }
    }
}

}  // namespace

extern "C" {

// nsteps forward-Euler steps of the O2 scheme in place on u (work: one more array of the same
// size). Same parameters as the oracle's heat calls; order 2 and no periodic wrap only.
void orc_cpu_heat_euler_o2_f32(int ndim, int nx, int ny, int nz, int frozen, int zero_boundary, double kx, double ky,
                               double kz, double dt, int64_t nsteps, float* u, float* work) {
  const int64_t NZ = ndim == 3 ? nz : 1;
  float* a = u;
  float* b = work;
  for (int64_t s = 0; s < nsteps; ++s) {
    euler_o2_sweep<float>(ndim, nx, ny, NZ, frozen, zero_boundary, (float)kx, (float)ky, (float)kz, (float)dt, a, b);
    std::swap(a, b);
  }
  if (a != u) std::memcpy(u, a, sizeof(float) * (size_t)nx * ny * NZ);
}

}  // extern "C"
