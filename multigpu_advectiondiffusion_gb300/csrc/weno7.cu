// weno7.cu -- the seventh-order WENO Burgers solver of the reference's MATLAB prototypes on the GPU
// (Matlab_Prototipes/InviscidBurgersNd/WENO7resAdv_{X,Y,Z}.m, LFWENO7FDM{2,3}d.m:65-104).
//
// Scheme (per axis, on every line of the grid):
//   * local Lax-Friedrichs split f+- = (f +- |u| u)/2 of f = u^2/2 at every node;
//   * the line extended past its ends by copies of its end values (a clamped index), faces at
//     i+1/2 for i = 0..N-1, the face left of node 0 taken as 0;
//   * the seven-point WENO of Balsara & Shu (J. Comput. Phys. 160 (2000) 405-452): four cubic
//     candidates, linear weights 1/35, 12/35, 18/35, 4/35, weights d_k / (eps + beta_k)^2,
//     eps = 1e-6, the prototype's integer quadratic-form smoothness indicators
//     (WENO7resAdv_X.m:75-82);
//   * res_i = (((hp_{i+1/2} + hn_{i+1/2}) - hp_{i-1/2}) - hn_{i-1/2}) / h, summed over the axes in
//     axis order;
//   * time: dt = CFL dx / max|u| trimmed to land on tEnd, the five-stage fourth-order 2N-storage
//     Runge-Kutta scheme of Carpenter & Kennedy (NASA TM-109112, 1994): r = A_s r + dt R(u),
//     u = u - B_s r.
// For the FP64 state every operation is evaluated in the prototypes' operand order with correctly
// rounded intrinsics (no contraction), so its results are those of the prototypes -- and of the
// CPU oracle that restates them -- bit for bit; the FP32 state's faces take a faster form of the
// same scheme (the FP32 face kernels below).
//
// Kernels. Per stage and axis: a face kernel (one thread per face i+1/2, the two split parts'
// reconstructions hp and hn into two face arrays) and a residual kernel (one thread per node,
// accumulating the axis's residual into the stage's right-hand side); the last axis's residual
// kernel also applies the Runge-Kutta update in place and, at the last stage, reduces max|u| for
// the next step's dt. Threads run along x, so every access of every axis is coalesced. The time
// loop is one CUDA graph with a device-driven while node (the step-start kernel of the Burgers
// loop: dt rule, trim, t in FP64).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>

#include "adv_device.cuh"
#include "adv_internal.h"
#include "adv_math.cuh"
#include "nvtx_range.h"
#include "weno.cuh"

namespace adv {
namespace {

// Smoothness indicator of WENO7 candidate k over its cells x0..x3, in the prototype's order:
//   x2 (k0 x2 + k1 x3) + x0 (((k2 xb + k3 xc) + k4 xd) + k5 x3) + k6 x3 x3 + x1 ((k7 xs + k8 xt) + k9 x3)
// (the same table as the oracle's kW7Beta).
struct W7B {
  int b, c, d, s, t;
  double k[10];
};
__device__ constexpr W7B kBeta[4] = {
    {2, 1, 0, 2, 1, {134241, -114894, 56694, -47214, 6649, -22778, 25729, -210282, 85641, 86214}},
    {1, 0, 2, 1, 2, {41001, -30414, -19374, 3169, 19014, -5978, 6649, 33441, -70602, 23094}},
    {0, 1, 2, 1, 2, {33441, -19374, 6649, -30414, 23094, -5978, 3169, 41001, -70602, 19014}},
    {0, 1, 2, 1, 2, {85641, -47214, 25729, -114894, 86214, -22778, 6649, 134241, -210282, 56694}},
};
// candidates (c0 x0 + c1 x1 + c2 x2 + c3 x3)/12: the part moving towards +x (cells i-3+k .. i+k)
// and towards -x (cells i-2+k .. i+1+k); linear weights of each
__device__ constexpr double kPolyP[4][4] = {{-3, 13, -23, 25}, {1, -5, 13, 3}, {-1, 7, 7, -1}, {3, 13, -5, 1}};
__device__ constexpr double kPolyM[4][4] = {{1, -5, 13, 3}, {-1, 7, 7, -1}, {3, 13, -5, 1}, {25, -23, 13, -3}};
__device__ constexpr double kLinP[4] = {1. / 35., 12. / 35., 18. / 35., 4. / 35.};
__device__ constexpr double kLinM[4] = {4. / 35., 18. / 35., 12. / 35., 1. / 35.};

// Carpenter & Kennedy LSRK(5,4) coefficients (the published rational values).
__device__ constexpr double kA[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                                     -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
__device__ constexpr double kB[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                                     1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                                     2277821191437.0 / 14882151754819.0};

// One split part's face value from its seven cells f[0..6] (candidate k uses f[k..k+3]).
template <class T, bool PLUS>
__device__ __forceinline__ T weno7_part(const T (&f)[7]) {
  const T eps = T(1e-6);
  T a[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T* x = f + k;
    const W7B& B = kBeta[k];
    const T t1 = mul_rn(x[2], add_rn(mul_rn(T(B.k[0]), x[2]), mul_rn(T(B.k[1]), x[3])));
    const T t2 = mul_rn(x[0], add_rn(add_rn(add_rn(mul_rn(T(B.k[2]), x[B.b]), mul_rn(T(B.k[3]), x[B.c])),
                                            mul_rn(T(B.k[4]), x[B.d])),
                                     mul_rn(T(B.k[5]), x[3])));
    const T t3 = mul_rn(T(B.k[6]), mul_rn(x[3], x[3]));
    const T t4 = mul_rn(x[1], add_rn(add_rn(mul_rn(T(B.k[7]), x[B.s]), mul_rn(T(B.k[8]), x[B.t])),
                                     mul_rn(T(B.k[9]), x[3])));
    const T beta = add_rn(add_rn(add_rn(t1, t2), t3), t4);
    const T e = add_rn(eps, beta);
    a[k] = div_rn(T(PLUS ? kLinP[k] : kLinM[k]), mul_rn(e, e));
  }
  const T sum = add_rn(add_rn(add_rn(a[0], a[1]), a[2]), a[3]);
  T h = T(0);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T* x = f + k;
    const double* c = PLUS ? kPolyP[k] : kPolyM[k];
    const T cand = add_rn(add_rn(add_rn(mul_rn(T(c[0]), x[0]), mul_rn(T(c[1]), x[1])), mul_rn(T(c[2]), x[2])),
                          mul_rn(T(c[3]), x[3]));
    const T term = div_rn(mul_rn(div_rn(a[k], sum), cand), T(12));
    h = k == 0 ? term : add_rn(h, term);
  }
  return h;
}

// f+- of one node value (WENO7resAdv_X.m's split with a = |u|).
template <class T>
__device__ __forceinline__ void split(T v, T& fp, T& fm) {
  const T f = div_rn(mul_rn(v, v), T(2));
  const T av = mul_rn(fabs(v), v);
  fp = mul_rn(T(0.5), add_rn(f, av));
  fm = mul_rn(T(0.5), sub_rn(f, av));
}

struct W7Geom {
  int nx, ny, nz;
  int64_t n;
};

// Face kernel of axis AX: for every node (the face i+1/2 on its right along AX) the two parts'
// reconstructions into hp / hn.
template <class T, int AX>
__global__ void __launch_bounds__(256) weno7_face_kernel(const T* __restrict__ u, T* __restrict__ hp,
                                                         T* __restrict__ hn, W7Geom g) {
  const int64_t stride = AX == 0 ? 1 : AX == 1 ? (int64_t)g.nx : (int64_t)g.nx * g.ny;
  const int N = AX == 0 ? g.nx : AX == 1 ? g.ny : g.nz;
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < g.n; o += (int64_t)gridDim.x * blockDim.x) {
    const int64_t line_pos = AX == 0 ? o % g.nx : AX == 1 ? (o / g.nx) % g.ny : o / ((int64_t)g.nx * g.ny);
    const int i = (int)line_pos;
    const T* line = u + (o - (int64_t)i * stride);
    T fp[8], fm[8];  // cells i-3 .. i+4 (clamped)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int c = min(max(i + j - 3, 0), N - 1);
      split<T>(line[(int64_t)c * stride], fp[j], fm[j]);
    }
    T p[7], m[7];
#pragma unroll
    for (int j = 0; j < 7; ++j) {
      p[j] = fp[j];      // cells i-3 .. i+3
      m[j] = fm[j + 1];  // cells i-2 .. i+4
    }
    hn[o] = weno7_part<T, true>(p);
    hp[o] = weno7_part<T, false>(m);
  }
}

// ------------------------------------------------------------------ FP32 face kernels
// The FP32 state takes a form written for speed rather than the prototype's operand order (the
// FP64 state keeps that order, bit for bit):
//  * a tile of faces stages the split parts of its cells in shared memory once -- as 64-bit
//    pairs (f+ of a cell, f- of the next along the line), one load per operand pair -- instead of
//    every face re-reading and re-splitting its eight cells;
//  * both split parts of a face are reconstructed together in paired FP32 instructions (lane x
//    the part moving towards +x on cells i-3..i+3, lane y the other on cells i-2..i+4: the
//    smoothness indicators use the same coefficients on both);
//  * the prototype's weights d_k / (eps + beta_k)^2, normalised, are evaluated from
//    r_k = e_min / e_k (e_k = eps + beta_k, e_min the smallest): alpha_k = d_k r_k^2 lies in
//    (0, d_k] and the largest is at least d_min, so no product overflows, underflows or leaves a
//    zero sum, and the face value sum_k alpha_k q_k / (12 sum_k alpha_k) takes one division; the
//    quotients use the reciprocal-based division (at most 2 ulp each).
// Tiles: AX = 0, 32 faces along x by 8 rows (one face per thread); AX = 1, 2, 32 x positions by
// 32 faces along the line (four faces per thread). Cells past a line's ends are its end values
// (clamped), as in the prototype.
namespace w7f {
constexpr int TX = 32;  // x positions (AX = 0: faces) per tile
constexpr int TR = 8;   // rows per tile, AX = 0
constexpr int TL = 32;  // faces along the line per tile, AX = 1, 2
}  // namespace w7f

template <int K>
__device__ __forceinline__ float2 w7_beta2(const float2* x) {  // x: the candidate's cells 0..3
  constexpr W7B B = kBeta[K];
  auto c = [](double v) { return f2((float)v); };
  const float2 a = fma2(c(B.k[1]), x[3], mul2(c(B.k[0]), x[2]));
  const float2 b = fma2(c(B.k[5]), x[3], fma2(c(B.k[4]), x[B.d], fma2(c(B.k[3]), x[B.c], mul2(c(B.k[2]), x[B.b]))));
  const float2 t = fma2(c(B.k[9]), x[3], fma2(c(B.k[8]), x[B.t], mul2(c(B.k[7]), x[B.s])));
  return fma2(x[0], b, fma2(x[1], t, fma2(mul2(c(B.k[6]), x[3]), x[3], mul2(x[2], a))));
}

template <int K>
__device__ __forceinline__ float2 w7_cand2(const float2* x) {  // 12 x candidate K, per lane
  auto c = [](int j) { return make_float2((float)kPolyP[K][j], (float)kPolyM[K][j]); };
  return fma2(c(3), x[3], fma2(c(2), x[2], fma2(c(1), x[1], mul2(c(0), x[0]))));
}

// x[j] = (f+ of cell i-3+j, f- of cell i-2+j), j = 0..6. Returns (hn, hp): the +x part on cells
// i-3..i+3, the -x part on cells i-2..i+4.
__device__ __forceinline__ float2 w7_face2(const float2 (&x)[7]) {
  const float2 eps = f2(1e-6f);
  const float2 e0 = add2(w7_beta2<0>(x + 0), eps), e1 = add2(w7_beta2<1>(x + 1), eps);
  const float2 e2 = add2(w7_beta2<2>(x + 2), eps), e3 = add2(w7_beta2<3>(x + 3), eps);
  const float2 em = make_float2(fminf(fminf(e0.x, e1.x), fminf(e2.x, e3.x)), fminf(fminf(e0.y, e1.y), fminf(e2.y, e3.y)));
  auto alpha = [&](float2 e, int k) {
    const float2 r = make_float2(__fdividef(em.x, e.x), __fdividef(em.y, e.y));
    return mul2(mul2(make_float2((float)kLinP[k], (float)kLinM[k]), r), r);
  };
  const float2 a0 = alpha(e0, 0), a1 = alpha(e1, 1), a2 = alpha(e2, 2), a3 = alpha(e3, 3);
  const float2 num = fma2(a3, w7_cand2<3>(x + 3), fma2(a2, w7_cand2<2>(x + 2), fma2(a1, w7_cand2<1>(x + 1),
                                                                                   mul2(a0, w7_cand2<0>(x + 0)))));
  const float2 den = mul2(f2(12.f), add2(add2(a0, a1), add2(a2, a3)));
  return make_float2(__fdividef(num.x, den.x), __fdividef(num.y, den.y));
}

// (f+, f-) of one node value: f = u^2/2 split with a = |u|.
__device__ __forceinline__ float2 w7_split_fast(float v) {
  const float f = 0.5f * v * v, av = fabsf(v) * v;
  return make_float2(0.5f * (f + av), 0.5f * (f - av));
}

template <int AX>
__global__ void __launch_bounds__(256) weno7_face_fast_kernel(const float* __restrict__ u, float* __restrict__ hp,
                                                              float* __restrict__ hn, W7Geom g) {
  using namespace w7f;
  constexpr int ROWS = AX == 0 ? TR : TL + 7;  // shared rows: y rows (AX 0) or line cells
  constexpr int COLS = AX == 0 ? TX + 8 : TX;  // shared columns: x cells (AX 0; 39 used) or x
  __shared__ float2 fs[ROWS][COLS];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const int x0 = blockIdx.x * TX;
  // line position of the tile's first face and the fixed coordinate(s)
  const int l0 = AX == 0 ? x0 : blockIdx.y * TL;
  const int N = AX == 0 ? nx : AX == 1 ? ny : nz;
  const int64_t sxy = (int64_t)nx * ny;
  auto at = [&](int x, int y, int z) { return (int64_t)z * sxy + (int64_t)y * nx + x; };
  for (int e = threadIdx.x; e < ROWS * COLS; e += 256) {
    const int r = e / COLS, c = e - r * COLS;
    float2 v = make_float2(0.f, 0.f);
    if (AX == 0) {
      const int y = blockIdx.y * TR + r, z = blockIdx.z;
      const int x = min(max(x0 + c - 3, 0), nx - 1);
      if (c < TX + 7 && y < ny) v = w7_split_fast(u[at(x, y, z)]);
    } else {
      const int x = x0 + c, l = min(max(l0 + r - 3, 0), N - 1);
      if (x < nx) v = w7_split_fast(AX == 1 ? u[at(x, l, blockIdx.z)] : u[at(x, blockIdx.z, l)]);
    }
    // element t of a line holds (f+ of cell t, f- of cell t+1): the operand pairs of the paired
    // reconstruction, loaded as they are (18% faster than packing them from (f+, f-) per cell)
    float* fsf = reinterpret_cast<float*>(&fs[0][0]);
    fsf[2 * (r * COLS + c)] = v.x;
    if (AX == 0 ? c > 0 : r > 0) fsf[2 * (AX == 0 ? r * COLS + c - 1 : (r - 1) * COLS + c) + 1] = v.y;
  }
  __syncthreads();
  if (AX == 0) {
    const int x = x0 + tx, y = blockIdx.y * TR + ty;
    if (x < nx && y < ny) {
      float2 c[7];
#pragma unroll
      for (int j = 0; j < 7; ++j) c[j] = fs[ty][tx + j];
      const float2 h = w7_face2(c);
      const int64_t o = at(x, y, blockIdx.z);
      hn[o] = h.x;
      hp[o] = h.y;
    }
  } else {
    const int x = x0 + tx;
    if (x < nx) {
#pragma unroll
      for (int j = 0; j < TL / 8; ++j) {
        const int t = ty + 8 * j, l = l0 + t;
        if (l < N) {
          float2 c[7];
#pragma unroll
          for (int m = 0; m < 7; ++m) c[m] = fs[t + m][tx];
          const float2 h = w7_face2(c);
          const int64_t o = AX == 1 ? at(x, l, blockIdx.z) : at(x, blockIdx.z, l);
          hn[o] = h.x;
          hp[o] = h.y;
        }
      }
    }
  }
}

// Face launch of axis AX: the tiled FP32 kernel where its grid fits, else the generic kernel.
template <class T, int AX>
void weno7_face_launch(const T* u, T* hp, T* hn, const W7Geom& g, int grid, cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value) {
    using namespace w7f;
    const int64_t gx = (g.nx + TX - 1) / TX;
    const int64_t gy = AX == 0 ? (g.ny + TR - 1) / TR : AX == 1 ? (g.ny + TL - 1) / TL : (g.nz + TL - 1) / TL;
    const int64_t gz = AX == 2 ? g.ny : g.nz;
    if (gx <= 0x7fffffff && gy <= 65535 && gz <= 65535) {
      weno7_face_fast_kernel<AX><<<dim3((unsigned)gx, (unsigned)gy, (unsigned)gz), 256, 0, s>>>(u, hp, hn, g);
      return;
    }
  }
  weno7_face_kernel<T, AX><<<grid, 256, 0, s>>>(u, hp, hn, g);
}

// Residual kernel of axis AX: res_i = (((hp_i + hn_i) - hp_{i-1}) - hn_{i-1}) / h (0 for the face
// left of node 0), accumulated into acc (FIRST: acc = res). LAST: then the Runge-Kutta update
// r = A r + dt acc, u = u - B r in place, and (REDUCE) max|u_new| into *maxkey.
constexpr int kW7ResZ = 16;  // z planes per thread of the tiled residual kernel

// TILED: a 3D grid of 32 x 8 (x, y) tiles, each thread walking kW7ResZ z planes of its column,
// so a node's line position comes from its coordinates; otherwise a grid-stride loop over the
// flat index (whose line position takes an integer division).
template <class T, int AX, bool FIRST, bool LAST, bool TILED>
__global__ void __launch_bounds__(256) weno7_residual_kernel(const T* __restrict__ hp, const T* __restrict__ hn,
                                                             T* __restrict__ acc, T* __restrict__ r, T* __restrict__ u,
                                                             W7Geom g, T h, int stage, const double* dt_dev,
                                                             typename KeyOf<T>::type* maxkey, const int* active) {
  using K = typename KeyOf<T>::type;
  if (active && *active == 0) return;
  const int64_t stride = AX == 0 ? 1 : AX == 1 ? (int64_t)g.nx : (int64_t)g.nx * g.ny;
  const T A = T(kA[stage]), B = T(kB[stage]);
  const T dt = LAST ? T(*dt_dev) : T(0);
  K kmax = 0;
  int64_t o, o_end, o_step;
  int64_t i = 0;
  if (TILED) {
    const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
    const int z0 = blockIdx.z * kW7ResZ, z1 = min(g.nz, z0 + kW7ResZ);
    const bool in = x < g.nx && y < g.ny;
    o_step = (int64_t)g.nx * g.ny;
    o = (int64_t)z0 * o_step + (int64_t)y * g.nx + x;
    o_end = in ? o + (int64_t)(z1 - z0) * o_step : o;
    i = AX == 0 ? x : AX == 1 ? y : z0;
  } else {
    o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    o_end = g.n;
    o_step = (int64_t)gridDim.x * blockDim.x;
  }
  for (; o < o_end; o += o_step, i += (TILED && AX == 2) ? 1 : 0) {
    if (!TILED) i = AX == 0 ? o % g.nx : AX == 1 ? (o / g.nx) % g.ny : o / ((int64_t)g.nx * g.ny);
    const T hp0 = i > 0 ? hp[o - stride] : T(0), hn0 = i > 0 ? hn[o - stride] : T(0);
    const T res = div_rn(sub_rn(sub_rn(add_rn(hp[o], hn[o]), hp0), hn0), h);
    const T L = FIRST ? res : add_rn(acc[o], res);
    if (!LAST) {
      acc[o] = L;
    } else {
      const T rn = add_rn(mul_rn(A, r[o]), mul_rn(dt, L));
      r[o] = rn;
      const T un = sub_rn(u[o], mul_rn(B, rn));
      u[o] = un;
      if (maxkey) {
        const K k = abs_key(un);
        kmax = k > kmax ? k : kmax;
      }
    }
  }
  if (LAST && maxkey) {
    kmax = warp_max(kmax);
    if ((threadIdx.x & 31) == 0 && kmax) atomicMax(maxkey, kmax);
  }
}

// Residual launch of axis AX: the tiled kernel where its grid fits, else the grid-stride one.
template <class T, int AX, bool FIRST, bool LAST>
void weno7_residual_launch(const T* hp, const T* hn, T* acc, T* r, T* u, const W7Geom& g, T h, int stage,
                           const double* dt_dev, typename KeyOf<T>::type* maxkey, const int* active, int grid,
                           cudaStream_t s) {
  const int64_t gx = (g.nx + 31) / 32, gy = (g.ny + 7) / 8, gz = (g.nz + kW7ResZ - 1) / kW7ResZ;
  if (gx <= 0x7fffffff && gy <= 65535 && gz <= 65535)
    weno7_residual_kernel<T, AX, FIRST, LAST, true><<<dim3((unsigned)gx, (unsigned)gy, (unsigned)gz), 256, 0, s>>>(
        hp, hn, acc, r, u, g, h, stage, dt_dev, maxkey, active);
  else
    weno7_residual_kernel<T, AX, FIRST, LAST, false><<<grid, 256, 0, s>>>(hp, hn, acc, r, u, g, h, stage, dt_dev,
                                                                          maxkey, active);
}

adv_status weno7_validate(const adv_weno7_desc* d) {
  if (!d) return set_error(ADV_ERR_INVALID_ARG, "weno7: null descriptor");
  if (d->dtype != ADV_F32 && d->dtype != ADV_F64) return set_error(ADV_ERR_INVALID_ARG, "weno7: bad dtype");
  if (d->nx < 1 || d->ny < 1 || d->nz < 1) return set_error(ADV_ERR_INVALID_ARG, "weno7: empty grid");
  if (d->ny < 2) return set_error(ADV_ERR_UNSUPPORTED, "weno7: 2D and 3D grids only (ny >= 2)");
  if ((int64_t)d->nx * d->ny * d->nz > ((int64_t)1 << 36)) return set_error(ADV_ERR_INVALID_ARG, "weno7: grid too large");
  if (!(d->dx > 0) || !(d->dy > 0) || !(d->dz > 0)) return set_error(ADV_ERR_INVALID_ARG, "weno7: spacing must be > 0");
  return ADV_OK;
}

size_t weno7_array_bytes(const adv_weno7_desc& d) {
  const size_t n = (size_t)d.nx * d.ny * d.nz;
  return (n * (d.dtype == ADV_F32 ? 4 : 8) + 255) / 256 * 256;
}

int weno7_ndim(const adv_weno7_desc& d) { return d.nz > 1 ? 3 : 2; }

// Workspace: hp, hn, acc, r, then the loop state.
struct W7Work {
  char *hp, *hn, *acc, *r;
  BurgersLoopState* st;
};
W7Work weno7_work(const adv_weno7_desc& d, void* ws) {
  const size_t one = weno7_array_bytes(d);
  char* b = static_cast<char*>(ws);
  return W7Work{b, b + one, b + 2 * one, b + 3 * one, reinterpret_cast<BurgersLoopState*>(b + 4 * one)};
}

int weno7_grid(const adv_weno7_desc& d) {
  DeviceInfo di;
  const int sms = device_info(&di) == ADV_OK ? di.sms : 152;
  const int64_t n = (int64_t)d.nx * d.ny * d.nz;
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 16));
}

// The face + residual launches of one stage (stage 0..4), the update fused into the last axis.
template <class T>
adv_status weno7_stage_t(const adv_weno7_desc& d, T* u, const W7Work& w, int stage, const double* dt_dev,
                         void* maxkey, const int* active, bool count, cudaStream_t s) {
  using K = typename KeyOf<T>::type;
  const W7Geom g{d.nx, d.ny, d.nz, (int64_t)d.nx * d.ny * d.nz};
  const int grid = weno7_grid(d);
  const int nd = weno7_ndim(d);
  T* hp = reinterpret_cast<T*>(w.hp);
  T* hn = reinterpret_cast<T*>(w.hn);
  T* acc = reinterpret_cast<T*>(w.acc);
  T* r = reinterpret_cast<T*>(w.r);
  K* mk = static_cast<K*>(maxkey);
  const T hx = T(d.dx), hy = T(d.dy), hz = T(d.dz);
  weno7_face_launch<T, 0>(u, hp, hn, g, grid, s);
  weno7_residual_launch<T, 0, true, false>(hp, hn, acc, r, u, g, hx, stage, dt_dev, mk, active, grid, s);
  weno7_face_launch<T, 1>(u, hp, hn, g, grid, s);
  if (nd == 2) {
    weno7_residual_launch<T, 1, false, true>(hp, hn, acc, r, u, g, hy, stage, dt_dev, mk, active, grid, s);
  } else {
    weno7_residual_launch<T, 1, false, false>(hp, hn, acc, r, u, g, hy, stage, dt_dev, mk,
                                                                   active, grid, s);
    weno7_face_launch<T, 2>(u, hp, hn, g, grid, s);
    weno7_residual_launch<T, 2, false, true>(hp, hn, acc, r, u, g, hz, stage, dt_dev, mk, active, grid, s);
  }
  ADV_CUDA_TRY(cudaGetLastError());
  if (count) count_launches(2 * nd);
  return ADV_OK;
}

adv_status weno7_stage(const adv_weno7_desc& d, void* u, const W7Work& w, int stage, const double* dt_dev,
                       void* maxkey, const int* active, bool count, cudaStream_t s) {
  if (d.dtype == ADV_F32)
    return weno7_stage_t<float>(d, static_cast<float*>(u), w, stage, dt_dev, maxkey, active, count, s);
  return weno7_stage_t<double>(d, static_cast<double*>(u), w, stage, dt_dev, maxkey, active, count, s);
}

// The right-hand side alone (the summed residuals, no update): RHS kernels into acc, then copied
// to the caller's L.
template <class T>
adv_status weno7_rhs_t(const adv_weno7_desc& d, const T* u, T* L, const W7Work& w, cudaStream_t s) {
  const W7Geom g{d.nx, d.ny, d.nz, (int64_t)d.nx * d.ny * d.nz};
  const int grid = weno7_grid(d);
  const int nd = weno7_ndim(d);
  T* hp = reinterpret_cast<T*>(w.hp);
  T* hn = reinterpret_cast<T*>(w.hn);
  weno7_face_launch<T, 0>(u, hp, hn, g, grid, s);
  weno7_residual_launch<T, 0, true, false>(hp, hn, L, nullptr, nullptr, g, T(d.dx), 0, nullptr,
                                                                 nullptr, nullptr, grid, s);
  weno7_face_launch<T, 1>(u, hp, hn, g, grid, s);
  weno7_residual_launch<T, 1, false, false>(hp, hn, L, nullptr, nullptr, g, T(d.dy), 0, nullptr,
                                                                 nullptr, nullptr, grid, s);
  if (nd == 3) {
    weno7_face_launch<T, 2>(u, hp, hn, g, grid, s);
    weno7_residual_launch<T, 2, false, false>(hp, hn, L, nullptr, nullptr, g, T(d.dz), 0,
                                                                   nullptr, nullptr, nullptr, grid, s);
  }
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(2 * nd);
  return ADV_OK;
}

}  // namespace
}  // namespace adv

using namespace adv;

extern "C" {

adv_status adv_weno7_workspace_bytes(const adv_weno7_desc* d, size_t* bytes) {
  adv_status st = weno7_validate(d);
  if (st != ADV_OK) return st;
  if (!bytes) return set_error(ADV_ERR_INVALID_ARG, "weno7: null output");
  *bytes = 4 * weno7_array_bytes(*d) + (sizeof(BurgersLoopState) + 255) / 256 * 256;
  return ADV_OK;
}

adv_status adv_weno7_rhs(const adv_weno7_desc* d, const void* u, void* L, void* workspace, void* stream) {
  ADV_NVTX_RANGE("adv_weno7_rhs");
  adv_status st = weno7_validate(d);
  if (st != ADV_OK) return st;
  if (!u || !L || !workspace) return set_error(ADV_ERR_INVALID_ARG, "weno7: null buffer");
  if (u == L) return set_error(ADV_ERR_INVALID_ARG, "weno7: u and L must not alias");
  const W7Work w = weno7_work(*d, workspace);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (d->dtype == ADV_F32) return weno7_rhs_t<float>(*d, static_cast<const float*>(u), static_cast<float*>(L), w, s);
  return weno7_rhs_t<double>(*d, static_cast<const double*>(u), static_cast<double*>(L), w, s);
}

adv_status adv_weno7_run(const adv_weno7_desc* d, void* u, void* workspace, double tEnd, double cfl,
                         int64_t max_steps, double* t_out, int64_t* steps_out, void* stream) {
  ADV_NVTX_RANGE("adv_weno7_run");
  adv_status st = weno7_validate(d);
  if (st != ADV_OK) return st;
  if (!u || !workspace) return set_error(ADV_ERR_INVALID_ARG, "weno7: null buffer");
  if (!(cfl > 0) || !std::isfinite(tEnd) || max_steps < 0) return set_error(ADV_ERR_INVALID_ARG, "weno7: bad cfl/tEnd/max_steps");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if ((st = reject_capture(s, "weno7 run")) != ADV_OK) return st;
  const W7Work w = weno7_work(*d, workspace);
  const size_t n = (size_t)d->nx * d->ny * d->nz;
  const size_t es = d->dtype == ADV_F32 ? 4 : 8;
  // loop state: the Burgers loop's dt rule MAXU (dt = CFL dx / max|u|, trimmed to tEnd)
  adv_burgers_desc bd{};
  bd.nx = d->nx; bd.ny = d->ny; bd.nz = d->nz;
  bd.dx = d->dx; bd.dy = d->dy; bd.dz = d->dz;
  BurgersLoopState h = burgers_loop_state(bd, tEnd, cfl, ADV_DT_MAXU, 0.0, max_steps);
  ADV_CUDA_TRY(cudaMemcpyAsync(w.st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  ADV_CUDA_TRY(cudaMemsetAsync(w.r, 0, n * es, s));  // the 2N-storage register starts at zero
  void* key0 = d->dtype == ADV_F32 ? (void*)&w.st->maxbits[0] : (void*)&w.st->maxbits64[0];
  if ((st = max_abs_launch(d->dtype, u, (int64_t)n, key0, s)) != ADV_OK) return st;
  // one time step: the step-start kernel (dt, t, loop condition), then five stages; the last one
  // reduces max|u| for the next step into slot 0
  const int nd = weno7_ndim(*d);
  auto body = [&](cudaStream_t cs, unsigned long long cond, int use_cond) -> adv_status {
    adv_status r = burgers_loop_begin_step(w.st, d->dtype, cond, use_cond, cs);
    for (int stg = 0; stg < 5 && r == ADV_OK; ++stg)
      r = weno7_stage(*d, u, w, stg, &w.st->dt, stg == 4 ? key0 : nullptr, &w.st->active, !use_cond, cs);
    return r;
  };
  const int64_t launched_per_step = 1 + 5 * 2 * nd;
  bool graph_ran = false;
  if (max_steps > 0 && tEnd > 0.0) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    cudaStream_t cs;
    ADV_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaError_t e = cudaGraphCreate(&g, 0);
    cudaGraphConditionalHandle h_cond = 0;
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h_cond, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNode_t node;
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h_cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
    adv_status bst = ADV_OK;
    if (e == cudaSuccess) {
      e = cudaStreamBeginCaptureToGraph(cs, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        bst = body(cs, (unsigned long long)h_cond, 1);
        cudaGraph_t outg = nullptr;
        e = cudaStreamEndCapture(cs, &outg);
      }
      if (e == cudaSuccess && bst == ADV_OK) e = cudaGraphInstantiate(&ge, g, 0);
    }
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (bst != ADV_OK) {
      if (ge) cudaGraphExecDestroy(ge);
      return bst;
    }
    if (e == cudaSuccess && ge) {
      graph_ran = true;
      e = cudaGraphLaunch(ge, s);
      cudaError_t e2 = cudaStreamSynchronize(s);
      cudaGraphExecDestroy(ge);
      if (e != cudaSuccess) return cuda_error(e, "weno7: graph launch");
      if (e2 != cudaSuccess) return cuda_error(e2, "weno7: run");
    } else {
      cudaGetLastError();  // conditional nodes unavailable: one step at a time from the host
      if (ge) cudaGraphExecDestroy(ge);
      for (int64_t i = 0; i < max_steps; ++i) {
        if ((st = body(s, 0, 0)) != ADV_OK) return st;
        int active = 0;
        ADV_CUDA_TRY(cudaMemcpyAsync(&active, &w.st->active, sizeof(int), cudaMemcpyDeviceToHost, s));
        ADV_CUDA_TRY(cudaStreamSynchronize(s));
        if (!active) break;
      }
    }
  }
  ADV_CUDA_TRY(cudaMemcpyAsync(&h, w.st, sizeof(h), cudaMemcpyDeviceToHost, s));
  ADV_CUDA_TRY(cudaStreamSynchronize(s));
  if (graph_ran) count_launches(launched_per_step * h.step);  // (the host loop counted its own)
  if (t_out) *t_out = h.t;
  if (steps_out) *steps_out = h.step;
  return read_and_clear_device_status(s);
}

}  // extern "C"
