// heat2d_multi.cu -- 2D forward-Euler heat, several time steps per launch (overlapped temporal
// tiling) for adv_heat_run.
//
// A 2D grid of the reference's sizes (SingleGPU/Diffusion2d: 512^2 .. 1001^2 nodes, 1-4 MB per
// array) is too small to hide a launch per step: the single-step stage spends most of its time
// in launch gaps and in the load -> compute -> store latency of one plane. Here a CTA copies a
// 32 x 32 tile of outputs plus a halo of K * R nodes (R the stencil radius) into shared memory
// once, advances it K steps in place -- after step s the values are valid on the tile grown by
// (K - s) * R, so the halo's recomputation shrinks step by step -- and writes the tile once:
// one launch and one pass over memory per K steps (FP32; in FP64 the recomputed halo costs more on
// the FP64 pipe than the launches it saves, so FP64 keeps one step per launch). Each node's
// update is the fused single-step
// stage's expression (lap / combine of heat_stage.cuh, the fused multiply-add form), applied to
// the same neighbour values, so the result equals K single steps bit for bit.
#include <algorithm>

#include "adv_device.cuh"
#include "adv_internal.h"
#include "heat_stage.cuh"

namespace adv {

struct Heat2Multi {
  static constexpr int BX = 32, BY = 32;  // outputs per CTA
  static constexpr int K = 8;             // steps per launch at most (4: 118, 16: 138 Gcell/s)
  static constexpr int TX = 32, TY = 16;  // 512 threads (256: 122 vs 145 Gcell/s at 512^2)
};

template <class T>
struct Heat2MultiParams {
  const T* in;
  T* out;
  int nx, ny, frozen, zero_boundary, steps;
  T kx, ky, dt;
  int* status;  // device status word (bounds-checked build)
};

template <class T, int ORDER, bool FAST>
__global__ void __launch_bounds__(512) heat2d_multi_kernel(const __grid_constant__ Heat2MultiParams<T> p) {
  using M = Heat2Multi;
  constexpr int R = ORDER / 2, H = M::K * R;
  constexpr int EX = M::BX + 2 * H, EY = M::BY + 2 * H;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* bufA = reinterpret_cast<T*>(smem_raw);
  T* bufB = bufA + EX * EY;
  const int x0 = blockIdx.x * M::BX - H, y0 = blockIdx.y * M::BY - H;  // grid coordinates of buffer (0, 0)
  const int nx = p.nx, ny = p.ny, F = p.frozen;
  // load the grown tile (nodes off the grid read as 0; no update ever reads them)
  for (int j = threadIdx.y; j < EY; j += M::TY) {
    const int gy = y0 + j;
    for (int i = threadIdx.x; i < EX; i += M::TX) {
      const int gx = x0 + i;
      const size_t gi = (size_t)gy * nx + gx;
      bufA[j * EX + i] = (gx >= 0 && gx < nx && gy >= 0 && gy < ny && ADV_IN_RANGE(gi, (size_t)nx * ny, p.status))
                             ? p.in[gi]
                             : T(0);
    }
  }
  __syncthreads();
  T* src = bufA;
  T* dst = bufB;
  // Every step updates the whole buffer but its outer R nodes with the interior formula, without
  // per-node domain tests: values that are no longer valid after step s (a ring that grows by R
  // per step), and values of nodes off the grid, are never read by a valid interior node (those
  // are at least F >= R nodes inside the grid). Frozen nodes of the grid then take their own rule
  // (kept, or 0 on the outermost layer with zero_boundary); only CTAs whose grown tile reaches
  // into the frozen layers test for them.
  const bool inner = x0 >= F && x0 + EX <= nx - F && y0 >= F && y0 + EY <= ny - F;
  const bool zero = p.zero_boundary != 0;
  for (int s = 1; s <= p.steps; ++s) {
    for (int j = R + threadIdx.y; j < EY - R; j += M::TY) {
      const int gy = y0 + j;
      const bool rowF = gy < F || gy >= ny - F, rowO = gy == 0 || gy == ny - 1;
      const T* row = src + j * EX;
      T* drow = dst + j * EX;
      for (int i = R + threadIdx.x; i < EX - R; i += M::TX) {
        const T* c = row + i;
        const T L = lap<T, ORDER, 2, FAST>(R > 1 ? c[-2] : T(0), c[-1], c[0], c[1], R > 1 ? c[2] : T(0),
                                           R > 1 ? c[-2 * EX] : T(0), c[-EX], c[EX], R > 1 ? c[2 * EX] : T(0),
                                           T(0), T(0), T(0), T(0), p.kx, p.ky, T(0));
        T v = combine<T, FAST>(1, c[0], c[0], p.dt, L);
        if (!inner) {
          const int gx = x0 + i;
          if (rowF || gx < F || gx >= nx - F) v = (zero && (rowO || gx == 0 || gx == nx - 1)) ? T(0) : c[0];
        }
        drow[i] = v;
      }
    }
    __syncthreads();
    T* t = src;
    src = dst;
    dst = t;
  }
  // the tile itself
  for (int j = threadIdx.y; j < M::BY; j += M::TY) {
    const int gy = y0 + H + j;
    if (gy >= ny) break;
    for (int i = threadIdx.x; i < M::BX; i += M::TX) {
      const int gx = x0 + H + i;
      if (gx < nx && ADV_IN_RANGE((size_t)gy * nx + gx, (size_t)nx * ny, p.status))
        p.out[(size_t)gy * nx + gx] = src[(j + H) * EX + i + H];
    }
  }
}

namespace {
template <class T, int ORDER, bool FAST>
constexpr size_t heat2d_multi_smem() {
  constexpr int H = Heat2Multi::K * (ORDER / 2);
  return 2 * (size_t)(Heat2Multi::BX + 2 * H) * (Heat2Multi::BY + 2 * H) * sizeof(T);
}

template <class T, int ORDER, bool FAST>
adv_status launch_t(const adv_heat_desc& d, const void* in, void* out, int steps, cudaStream_t s) {
  constexpr size_t smem = heat2d_multi_smem<T, ORDER, FAST>();
  static bool attr = false;  // 18 KB (O2) or 32 KB (O4) per CTA: under the default 48 KB, set anyway
  if (!attr) {
    ADV_CUDA_TRY(cudaFuncSetAttribute(heat2d_multi_kernel<T, ORDER, FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    attr = true;
  }
  Heat2MultiParams<T> p;
  p.in = static_cast<const T*>(in);
  p.out = static_cast<T*>(out);
  p.nx = d.nx;
  p.ny = d.ny;
  p.frozen = d.frozen;
  p.zero_boundary = d.zero_boundary;
  p.steps = steps;
  p.kx = (T)d.kx;
  p.ky = (T)d.ky;
  p.dt = (T)d.dt;
  p.status = device_status_ptr();
  const dim3 grid((unsigned)((d.nx + Heat2Multi::BX - 1) / Heat2Multi::BX),
                  (unsigned)((d.ny + Heat2Multi::BY - 1) / Heat2Multi::BY));
  heat2d_multi_kernel<T, ORDER, FAST><<<grid, dim3(Heat2Multi::TX, Heat2Multi::TY), smem, s>>>(p);
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}
}  // namespace

int heat2d_multi_steps() { return Heat2Multi::K; }

adv_status heat2d_multi_launch(const adv_heat_desc& d, const void* in, void* out, int steps, cudaStream_t s) {
  if (d.ndim != 2 || steps < 1 || steps > Heat2Multi::K || in == out)
    return set_error(ADV_ERR_INVALID_ARG, "heat2d multi-step: bad arguments");
  if (d.dtype != ADV_F32) return set_error(ADV_ERR_UNSUPPORTED, "heat2d multi-step: FP32 only");
  return d.order == 2 ? launch_t<float, 2, true>(d, in, out, steps, s) : launch_t<float, 4, true>(d, in, out, steps, s);
}

}  // namespace adv
