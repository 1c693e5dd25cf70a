// ref_ops.cu -- the reference's unfused operators (include/advdiff_ref_ops.h) as sm_103a kernels.
//
// One thread per node, grid-stride over a flat index, so the launch never depends on the
// caller's block shape (the reference's wrappers take dim3 arguments; the compatibility
// libraries ignore them). Arithmetic uses correctly rounded intrinsics in the reference's
// operand order, so FP64 results equal the reference's own kernels' and the CPU oracle's.
#include <algorithm>

#include "../../include/advdiff_ref_ops.h"
#include "adv_device.cuh"
#include "adv_internal.h"
#include "nvtx_range.h"
#include "adv_math.cuh"
#include "weno.cuh"

namespace adv {

struct Grid3 {
  int nx, ny, nz;
  int64_t pitch;
  __device__ __forceinline__ int64_t count() const { return (int64_t)nx * ny * nz; }
  __device__ __forceinline__ void ijk(int64_t f, int& i, int& j, int& k) const {
    i = (int)(f % nx);
    const int64_t r = f / nx;
    j = (int)(r % ny);
    k = (int)(r / ny);
  }
  __device__ __forceinline__ int64_t at(int i, int j, int k) const { return i + pitch * j + pitch * ny * (int64_t)k; }
  __device__ __forceinline__ int64_t total() const { return pitch * ny * (int64_t)nz; }  // elements addressed
  int* st;  // device status word (bounds-checked build)
};

// Nodes a Laplacian writes: i in [i0, i1), j in [j0, j1), k in [k0, k1).
struct Box3 {
  int i0, i1, j0, j1, k0, k1;
};

// west_first: the O4 operand order of the 2D kernel (west/south/bottom neighbours first), which
// SG/Diffusion3d_Blocking/kernels.cu:66-68 and 78-80 also use in 3D; otherwise 3D takes the
// baseline's east-first order.
template <class T>
__global__ void ref_laplace_kernel(Grid3 g, int ndim, int order, Box3 b, int zero_outside, int west_first, T kx, T ky,
                                   T kz, const T* __restrict__ u, T* __restrict__ Lu) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < g.count(); f += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    g.ijk(f, i, j, k);
    const int64_t o = g.at(i, j, k);
    const bool in = i >= b.i0 && i < b.i1 && j >= b.j0 && j < b.j1 && k >= b.k0 && k < b.k1;
    if (!in) {
      if (zero_outside && ADV_IN_RANGE(o, g.total(), g.st)) Lu[o] = T(0);
      continue;
    }
    const int64_t sy = g.pitch, sz = g.pitch * g.ny;
    const int64_t span = (int64_t)(order / 2) * (ndim == 3 ? sz : sy);  // the stencil's farthest reach
    if (!ADV_IN_RANGE(o - span, g.total(), g.st) || !ADV_IN_RANGE(o + span, g.total(), g.st)) continue;
    const T c = u[o];
    T L;
    if (order == 4) {
      if (ndim == 3 && west_first) {
        const T Sx = sub_rn(add_rn(sub_rn(add_rn(-u[o - 2], mul_rn(T(16), u[o - 1])), mul_rn(T(30), c)), mul_rn(T(16), u[o + 1])), u[o + 2]);
        const T Sy = sub_rn(add_rn(sub_rn(add_rn(-u[o - 2 * sy], mul_rn(T(16), u[o - sy])), mul_rn(T(30), c)), mul_rn(T(16), u[o + sy])), u[o + 2 * sy]);
        const T Sz = sub_rn(add_rn(sub_rn(add_rn(-u[o - 2 * sz], mul_rn(T(16), u[o - sz])), mul_rn(T(30), c)), mul_rn(T(16), u[o + sz])), u[o + 2 * sz]);
        L = add_rn(add_rn(mul_rn(kx, Sx), mul_rn(ky, Sy)), mul_rn(kz, Sz));
      } else if (ndim == 3) {  // east first (Diffusion3d_baselineCode/kernels.cu:95-97)
        const T Sx = sub_rn(add_rn(sub_rn(add_rn(-u[o + 2], mul_rn(T(16), u[o + 1])), mul_rn(T(30), c)), mul_rn(T(16), u[o - 1])), u[o - 2]);
        const T Sy = sub_rn(add_rn(sub_rn(add_rn(-u[o + 2 * sy], mul_rn(T(16), u[o + sy])), mul_rn(T(30), c)), mul_rn(T(16), u[o - sy])), u[o - 2 * sy]);
        const T Sz = sub_rn(add_rn(sub_rn(add_rn(-u[o + 2 * sz], mul_rn(T(16), u[o + sz])), mul_rn(T(30), c)), mul_rn(T(16), u[o - sz])), u[o - 2 * sz]);
        L = add_rn(add_rn(mul_rn(kx, Sx), mul_rn(ky, Sy)), mul_rn(kz, Sz));
      } else {  // west first (Diffusion2d/kernels.cu:82-83)
        const T Sx = sub_rn(add_rn(sub_rn(add_rn(-u[o - 2], mul_rn(T(16), u[o - 1])), mul_rn(T(30), c)), mul_rn(T(16), u[o + 1])), u[o + 2]);
        const T Sy = sub_rn(add_rn(sub_rn(add_rn(-u[o - 2 * sy], mul_rn(T(16), u[o - sy])), mul_rn(T(30), c)), mul_rn(T(16), u[o + sy])), u[o + 2 * sy]);
        L = add_rn(mul_rn(kx, Sx), mul_rn(ky, Sy));
      }
    } else {  // 12*k*(e - 2o + w) per axis (kernels.cu:58-60)
      const T Sx = add_rn(sub_rn(u[o + 1], mul_rn(T(2), c)), u[o - 1]);
      const T Sy = add_rn(sub_rn(u[o + sy], mul_rn(T(2), c)), u[o - sy]);
      L = add_rn(mul_rn(mul_rn(T(12), kx), Sx), mul_rn(mul_rn(T(12), ky), Sy));
      if (ndim == 3) {
        const T Sz = add_rn(sub_rn(u[o + sz], mul_rn(T(2), c)), u[o - sz]);
        L = add_rn(L, mul_rn(mul_rn(T(12), kz), Sz));
      }
    }
    Lu[o] = L;
  }
}

template <class T>
__global__ void ref_rk_kernel(Grid3 g, int ndim, int lo, int step, T dt, T* __restrict__ u, const T* __restrict__ uo,
                              const T* __restrict__ Lu) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < g.count(); f += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    g.ijk(f, i, j, k);
    bool in = i >= lo && i < g.nx - lo && j >= lo && j < g.ny - lo;
    if (ndim == 3) in = in && k >= lo && k < g.nz - lo;
    if (!in || step < 1 || step > 3) continue;
    const int64_t o = g.at(i, j, k);
    if (!ADV_IN_RANGE(o, g.total(), g.st)) continue;
    u[o] = stage_combine<T>(step, uo[o], u[o], dt, Lu[o]);
  }
}

// One directional sweep (Compute_dF / dG / dH, SG/Burgers3d_WENO5/kernels.cu:197-394): for every
// node with a in [2, na-4] along the axis and the other two indices in [3, n-4], the face flux
// F(a+1/2) from f+ at a-2..a+2 and f- at a-1..a+3 (local Lax-Friedrichs split), and
// Lu = -(F(a+1/2) - F(a-1/2)) / h (x: assigned; y, z: accumulated), with F(2-1/2) taken as 0.
// One thread per line walks a upwards as the reference's sweeps do: each face is reconstructed
// once (the previous one is kept in a register) and each node split once (a sliding window of six
// split values). Threads of a warp take neighbouring x positions for the y and z sweeps
// (coalesced); the x sweep's lines are rows, read through L1.
template <class T, bool Z>
__global__ void __launch_bounds__(256) ref_sweep_kernel(Grid3 g, int axis, T h, const T* __restrict__ u,
                                                        T* __restrict__ Lu) {
  const int na = axis == 0 ? g.nx : axis == 1 ? g.ny : g.nz;
  const int nb = axis == 0 ? g.ny : g.nx, nc = axis == 2 ? g.ny : g.nz;
  const int lb = nb - 6, lc = nc - 6;  // the other indices run over [3, n-4]
  if (na < 6 || lb <= 0 || lc <= 0) return;
  const int64_t s = axis == 0 ? 1 : axis == 1 ? g.pitch : g.pitch * g.ny;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)lb * lc;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int b = 3 + (int)(t % lb), c = 3 + (int)(t / lb);
    const int i = axis == 0 ? 0 : b, j = axis == 0 ? b : (axis == 1 ? 0 : c), k = axis == 2 ? 0 : c;
    const int64_t o0 = g.at(i, j, k);  // node a = 0 of this line
    T fp[6], fm[6];                    // split values of nodes a-2 .. a+3
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const T v = ADV_IN_RANGE(o0 + q * s, g.total(), g.st) ? u[o0 + q * s] : T(0);
      lf_split<T>(v, fabs(v), fp[q], fm[q]);
    }
    T fu_old = T(0);
    for (int a = 2; a <= na - 4; ++a) {
      const T fu = weno_face_ref<Z, T>(fp[0], fp[1], fp[2], fp[3], fp[4], fm[1], fm[2], fm[3], fm[4], fm[5]);
      const int64_t o = o0 + (int64_t)a * s;
      if (ADV_IN_RANGE(o, g.total(), g.st)) {
        if (axis == 0) Lu[o] = div_rn(-sub_rn(fu, fu_old), h);
        else Lu[o] = sub_rn(Lu[o], div_rn(sub_rn(fu, fu_old), h));
      }
      fu_old = fu;
#pragma unroll
      for (int q = 0; q < 5; ++q) {
        fp[q] = fp[q + 1];
        fm[q] = fm[q + 1];
      }
      if (a + 4 < na) {
        const int64_t oa = o0 + (int64_t)(a + 4) * s;
        const T v = ADV_IN_RANGE(oa, g.total(), g.st) ? u[oa] : T(0);
        lf_split<T>(v, fabs(v), fp[5], fm[5]);
      }
    }
  }
}

// The shared-memory program's sweeps (Compute_dF / dG / dH,
// SG/Burgers3d_WENO5_SharedMem/kernels.cu:212-405): every node of every line, u taken as 0 beyond
// both ends of the line, face a-1/2 from nodes a-3 .. a+2 (the same local Lax-Friedrichs split),
// the weights normalised by a reciprocal (RECIP form of weno_face_ref). One thread per line walks
// a upwards with a sliding window of six split values; each face is reconstructed once.
template <class T, bool Z>
__global__ void __launch_bounds__(256) ref_sweep_all_kernel(Grid3 g, int axis, T h, const T* __restrict__ u,
                                                            T* __restrict__ Lu) {
  const int na = axis == 0 ? g.nx : axis == 1 ? g.ny : g.nz;
  const int nb = axis == 0 ? g.ny : g.nx, nc = axis == 2 ? g.ny : g.nz;
  const int64_t s = axis == 0 ? 1 : axis == 1 ? g.pitch : g.pitch * g.ny;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)nb * nc;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(t % nb), c = (int)(t / nb);
    const int i = axis == 0 ? 0 : b, j = axis == 0 ? b : (axis == 1 ? 0 : c), k = axis == 2 ? 0 : c;
    const int64_t o0 = g.at(i, j, k);  // node a = 0 of this line
    auto split = [&](int a, T& p, T& m) {
      const T v = a >= 0 && a < na && ADV_IN_RANGE(o0 + (int64_t)a * s, g.total(), g.st) ? u[o0 + (int64_t)a * s] : T(0);
      lf_split<T>(v, fabs(v), p, m);
    };
    T fp[6], fm[6];  // split values of nodes a-3 .. a+2 (face a-1/2)
#pragma unroll
    for (int q = 0; q < 6; ++q) split(q - 3, fp[q], fm[q]);
    T f_left = weno_face_ref<Z, T, true>(fp[0], fp[1], fp[2], fp[3], fp[4], fm[1], fm[2], fm[3], fm[4], fm[5]);
    for (int a = 0; a < na; ++a) {
#pragma unroll
      for (int q = 0; q < 5; ++q) {
        fp[q] = fp[q + 1];
        fm[q] = fm[q + 1];
      }
      split(a + 3, fp[5], fm[5]);  // window: nodes a-2 .. a+3 (face a+1/2)
      const T f_right = weno_face_ref<Z, T, true>(fp[0], fp[1], fp[2], fp[3], fp[4], fm[1], fm[2], fm[3], fm[4], fm[5]);
      const int64_t o = o0 + (int64_t)a * s;
      if (ADV_IN_RANGE(o, g.total(), g.st)) {
        if (axis == 0) Lu[o] = div_rn(-sub_rn(f_right, f_left), h);
        else Lu[o] = sub_rn(Lu[o], div_rn(sub_rn(f_right, f_left), h));
      }
      f_left = f_right;
    }
  }
}

template <class T>
__global__ void ref_viscous_kernel(Grid3 g, T kx, T ky, T kz, int bug_b2, const T* __restrict__ u, T* __restrict__ Lu) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < g.count(); f += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    g.ijk(f, i, j, k);
    if (i < 3 || i > g.nx - 4 || j < 3 || j > g.ny - 4 || k < 3 || k > g.nz - 3) continue;
    const int64_t o = g.at(i, j, k), sy = g.pitch, sz = g.pitch * g.ny;
    if (!ADV_IN_RANGE(o - 2 * sz, g.total(), g.st) || !ADV_IN_RANGE(o + 2 * sz, g.total(), g.st)) continue;
    const T c = u[o];
    const T vx = sub_rn(add_rn(sub_rn(add_rn(-u[o - 2], mul_rn(T(16), u[o - 1])), mul_rn(T(30), c)), mul_rn(T(16), u[o + 1])), u[o + 2]);
    const T vy = sub_rn(add_rn(sub_rn(add_rn(-u[o - 2 * sy], mul_rn(T(16), u[o - sy])), mul_rn(T(30), c)), mul_rn(T(16), u[o + sy])), u[o + 2 * sy]);
    const T vz = sub_rn(add_rn(sub_rn(add_rn(-u[o - 2 * sz], mul_rn(T(16), u[o - sz])), mul_rn(T(30), c)), mul_rn(T(16), u[o + sz])), u[o + 2 * sz]);
    const T v = add_rn(add_rn(mul_rn(kx, vx), mul_rn(ky, vy)), mul_rn(kz, vz));
    T L = add_rn(Lu[o], v);
    if (bug_b2 && k >= 16 && k <= 18) L = add_rn(L, v);
    Lu[o] = L;
  }
}

static adv_status check_grid(int dtype, int64_t pitch, int nx, int ny, int nz, const void* a, const void* b) {
  if (dtype != ADV_F32 && dtype != ADV_F64) return set_error(ADV_ERR_INVALID_ARG, "ref op: bad dtype");
  if (nx < 1 || ny < 1 || nz < 1 || pitch < nx) return set_error(ADV_ERR_INVALID_ARG, "ref op: bad sizes or pitch");
  if (!a || !b) return set_error(ADV_ERR_INVALID_ARG, "ref op: null buffer");
  return ADV_OK;
}

static dim3 flat_grid(int64_t n) {
  DeviceInfo di;
  int sms = 148;
  if (device_info(&di) == ADV_OK) sms = di.sms;
  return dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 16)));
}

}  // namespace adv

using namespace adv;

extern "C" {

static adv_status ref_laplace_launch(int dtype, int ndim, int order, Box3 b, int zero_outside, int west_first,
                                     int64_t pitch, int nx, int ny, int nz, double kx, double ky, double kz,
                                     const void* u, void* Lu, void* stream) {
  Grid3 g{nx, ny, nz, pitch, device_status_ptr()};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const dim3 grid = flat_grid((int64_t)nx * ny * nz);
  if (dtype == ADV_F64)
    ref_laplace_kernel<double><<<grid, 256, 0, s>>>(g, ndim, order, b, zero_outside, west_first, kx, ky, kz,
                                                    (const double*)u, (double*)Lu);
  else
    ref_laplace_kernel<float><<<grid, 256, 0, s>>>(g, ndim, order, b, zero_outside, west_first, (float)kx, (float)ky,
                                                   (float)kz, (const float*)u, (float*)Lu);
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}

adv_status adv_ref_laplace(int dtype, int ndim, int order, int lo, int zero_outside, int64_t pitch, int nx, int ny, int nz,
                           double kx, double ky, double kz, const void* u, void* Lu, void* stream) {
  ADV_NVTX_RANGE("adv_ref_laplace");
  if (ndim == 2) nz = 1;
  adv_status st = check_grid(dtype, pitch, nx, ny, nz, u, Lu);
  if (st != ADV_OK) return st;
  if ((ndim != 2 && ndim != 3) || (order != 2 && order != 4) || lo < order / 2)
    return set_error(ADV_ERR_INVALID_ARG, "ref_laplace: bad ndim/order/lo");
  const Box3 b{lo, nx - lo, lo, ny - lo, ndim == 3 ? lo : 0, ndim == 3 ? nz - lo : 1};
  return ref_laplace_launch(dtype, ndim, order, b, zero_outside, 0, pitch, nx, ny, nz, kx, ky, kz, u, Lu, stream);
}

adv_status adv_ref_laplace_box(int dtype, int ndim, int order, const int32_t* box, int zero_outside, int west_first,
                               int64_t pitch, int nx, int ny, int nz, double kx, double ky, double kz, const void* u,
                               void* Lu, void* stream) {
  ADV_NVTX_RANGE("adv_ref_laplace_box");
  if (ndim == 2) nz = 1;
  adv_status st = check_grid(dtype, pitch, nx, ny, nz, u, Lu);
  if (st != ADV_OK) return st;
  if ((ndim != 2 && ndim != 3) || (order != 2 && order != 4) || !box || (west_first != 0 && west_first != 1))
    return set_error(ADV_ERR_INVALID_ARG, "ref_laplace_box: bad ndim/order/box/west_first");
  const int r = order / 2;
  Box3 b{box[0], box[1], box[2], box[3], ndim == 3 ? box[4] : 0, ndim == 3 ? box[5] : 1};
  // every stencil read stays on the grid: [i0, i1) within [r, nx - r), and so on
  if (b.i0 < r || b.i1 > nx - r || b.j0 < r || b.j1 > ny - r || (ndim == 3 && (b.k0 < r || b.k1 > nz - r)))
    return set_error(ADV_ERR_INVALID_ARG, "ref_laplace_box: box reaches past the stencil's margin");
  // 2D has one operand order (west first); west_first only selects the 3D one
  return ref_laplace_launch(dtype, ndim, order, b, zero_outside, west_first, pitch, nx, ny, nz, kx, ky, kz, u, Lu,
                            stream);
}

adv_status adv_ref_rk(int dtype, int ndim, int lo, int64_t pitch, int nx, int ny, int nz, int step, double dt, void* u,
                      const void* uo, const void* Lu, void* stream) {
  ADV_NVTX_RANGE("adv_ref_rk");
  if (ndim == 2) nz = 1;
  adv_status st = check_grid(dtype, pitch, nx, ny, nz, u, uo);
  if (st != ADV_OK) return st;
  if (!Lu || (ndim != 2 && ndim != 3) || lo < 0 || step < 1 || step > 3)
    return set_error(ADV_ERR_INVALID_ARG, "ref_rk: bad arguments");
  Grid3 g{nx, ny, nz, pitch, device_status_ptr()};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const dim3 grid = flat_grid((int64_t)nx * ny * nz);
  if (dtype == ADV_F64)
    ref_rk_kernel<double><<<grid, 256, 0, s>>>(g, ndim, lo, step, dt, (double*)u, (const double*)uo, (const double*)Lu);
  else
    ref_rk_kernel<float><<<grid, 256, 0, s>>>(g, ndim, lo, step, (float)dt, (float*)u, (const float*)uo, (const float*)Lu);
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}

adv_status adv_ref_burgers_sweep(int dtype, int axis, int weno, int64_t pitch, int nx, int ny, int nz, double h,
                                 const void* u, void* Lu, void* stream) {
  ADV_NVTX_RANGE("adv_ref_burgers_sweep");
  adv_status st = check_grid(dtype, pitch, nx, ny, nz, u, Lu);
  if (st != ADV_OK) return st;
  if (axis < 0 || axis > 2 || (weno != ADV_WENO5_JS && weno != ADV_WENO5_Z) || !(h != 0.0))
    return set_error(ADV_ERR_INVALID_ARG, "ref_burgers_sweep: bad arguments");
  Grid3 g{nx, ny, nz, pitch, device_status_ptr()};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nb = axis == 0 ? ny : nx, nc = axis == 2 ? ny : nz;
  const dim3 grid = flat_grid((int64_t)std::max(nb - 6, 1) * std::max(nc - 6, 1));  // one thread per line
  const bool z = weno == ADV_WENO5_Z;
  if (dtype == ADV_F64) {
    if (z) ref_sweep_kernel<double, true><<<grid, 256, 0, s>>>(g, axis, h, (const double*)u, (double*)Lu);
    else ref_sweep_kernel<double, false><<<grid, 256, 0, s>>>(g, axis, h, (const double*)u, (double*)Lu);
  } else {
    if (z) ref_sweep_kernel<float, true><<<grid, 256, 0, s>>>(g, axis, (float)h, (const float*)u, (float*)Lu);
    else ref_sweep_kernel<float, false><<<grid, 256, 0, s>>>(g, axis, (float)h, (const float*)u, (float*)Lu);
  }
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}

adv_status adv_ref_burgers_sweep_all(int dtype, int axis, int weno, int64_t pitch, int nx, int ny, int nz, double h,
                                     const void* u, void* Lu, void* stream) {
  ADV_NVTX_RANGE("adv_ref_burgers_sweep_all");
  adv_status st = check_grid(dtype, pitch, nx, ny, nz, u, Lu);
  if (st != ADV_OK) return st;
  if (axis < 0 || axis > 2 || (weno != ADV_WENO5_JS && weno != ADV_WENO5_Z) || !(h != 0.0))
    return set_error(ADV_ERR_INVALID_ARG, "ref_burgers_sweep_all: bad arguments");
  Grid3 g{nx, ny, nz, pitch, device_status_ptr()};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nb = axis == 0 ? ny : nx, nc = axis == 2 ? ny : nz;
  const dim3 grid = flat_grid((int64_t)nb * nc);  // one thread per line
  const bool z = weno == ADV_WENO5_Z;
  if (dtype == ADV_F64) {
    if (z) ref_sweep_all_kernel<double, true><<<grid, 256, 0, s>>>(g, axis, h, (const double*)u, (double*)Lu);
    else ref_sweep_all_kernel<double, false><<<grid, 256, 0, s>>>(g, axis, h, (const double*)u, (double*)Lu);
  } else {
    if (z) ref_sweep_all_kernel<float, true><<<grid, 256, 0, s>>>(g, axis, (float)h, (const float*)u, (float*)Lu);
    else ref_sweep_all_kernel<float, false><<<grid, 256, 0, s>>>(g, axis, (float)h, (const float*)u, (float*)Lu);
  }
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}

adv_status adv_ref_burgers_viscous(int dtype, int64_t pitch, int nx, int ny, int nz, double kx, double ky, double kz,
                                   int bug_b2, const void* u, void* Lu, void* stream) {
  ADV_NVTX_RANGE("adv_ref_burgers_viscous");
  adv_status st = check_grid(dtype, pitch, nx, ny, nz, u, Lu);
  if (st != ADV_OK) return st;
  Grid3 g{nx, ny, nz, pitch, device_status_ptr()};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const dim3 grid = flat_grid((int64_t)nx * ny * nz);
  if (dtype == ADV_F64)
    ref_viscous_kernel<double><<<grid, 256, 0, s>>>(g, kx, ky, kz, bug_b2, (const double*)u, (double*)Lu);
  else
    ref_viscous_kernel<float><<<grid, 256, 0, s>>>(g, (float)kx, (float)ky, (float)kz, bug_b2, (const float*)u, (float*)Lu);
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}

}  // extern "C"
