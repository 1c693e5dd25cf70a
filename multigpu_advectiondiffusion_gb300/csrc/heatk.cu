// heatk.cu -- 3D heat with a spatially varying diffusivity k(x), its discrete adjoint, and the
// checkpointed forward/backward runs (adv_heatk_* in advdiff.h). No reference counterpart: the
// reference's diffusivity is one constant C (SingleGPU/Diffusion3d_baselineCode/main.cpp:58-61).
//
// Scheme (conservative 7-point form, arithmetic face averages), for an interior node i and each
// axis a with neighbours p (+1) and m (-1):
//   k_p = (k_i + k_p)/2, k_m = (k_i + k_m)/2,  F_a = k_p (u_p - u_i) - k_m (u_i - u_m)
//   u'_i = u_i + c_x F_x + c_y F_y + c_z F_z,   c_a = dt / h_a^2
// The outermost layer is frozen (held, or set to 0 with zero_boundary).
//
// Adjoint of one step (J depends on u' through lam' = dJ/du'): with the masked adjoint
// mu_j = [j interior] lam'_j and P_i = [i interior or not zero_boundary],
//   lam_i  = P_i lam'_i + sum_a c_a sum_{j in nb_a(i)} k_ij (mu_j - mu_i)
//   dJ/dk_i += 1/2 sum_a c_a sum_{j in nb_a(i)} (u_j - u_i)(mu_i - mu_j)
// (each face coefficient k_ij = (k_i + k_j)/2 feeds half its derivative to each end). Neighbours
// outside the domain contribute nothing.
//
// Kernels: one thread per (x, y) column over a chunk of z planes, z neighbours from a register
// window, x/y neighbours from global loads that hit L1 (adjacent threads share them). Every
// operation is an explicit correctly rounded add/mul/fma, mirrored by the oracle.
#include <algorithm>
#include <cstring>
#include <initializer_list>

#include "adv_internal.h"
#include "nvtx_range.h"
#include "adv_math.cuh"

namespace adv {

namespace {

constexpr int KX = 32;  // block width; the height (4..16 threads) and the z planes per CTA are tunable

__device__ __forceinline__ float fma_k(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_k(double a, double b, double c) { return __fma_rn(a, b, c); }

template <class T>
struct HeatKArgs {
  const T* k;
  const T* u;    // forward: u^n; adjoint: u^n (the step's input)
  const T* lam;  // adjoint: lam^{n+1}
  T* out;        // forward: u^{n+1}; adjoint: lam^n
  T* grad;       // adjoint: dJ/dk accumulator
  int nx, ny, nz, zero_boundary;
  int zc;  // z planes per CTA
  T cx, cy, cz;
};

template <class T>
__global__ void __launch_bounds__(512) heatk_step_kernel(const __grid_constant__ HeatKArgs<T> a) {
  const int x = blockIdx.x * KX + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.nx || y >= a.ny) return;
  const int z0 = blockIdx.z * a.zc, z1 = min(a.nz, z0 + a.zc);
  const size_t sx = 1, sy = (size_t)a.nx, sz = (size_t)a.nx * a.ny;
  const bool col_in = x > 0 && x < a.nx - 1 && y > 0 && y < a.ny - 1;
  const T h = T(0.5);
  size_t o = (size_t)x + sy * y + sz * z0;
  T uc = a.u[o], kc = a.k[o];
  T um = z0 > 0 ? a.u[o - sz] : uc, km = z0 > 0 ? a.k[o - sz] : kc;
  for (int z = z0; z < z1; ++z, o += sz) {
    const T up = z + 1 < a.nz ? a.u[o + sz] : uc, kp = z + 1 < a.nz ? a.k[o + sz] : kc;
    T res;
    if (col_in && z > 0 && z < a.nz - 1) {
      auto flux = [&](T u_p, T u_m, T k_p, T k_m) {
        const T fp = mul_rn(h, add_rn(kc, k_p)), fm = mul_rn(h, add_rn(kc, k_m));
        return fma_k(fp, sub_rn(u_p, uc), -mul_rn(fm, sub_rn(uc, u_m)));
      };
      const T Fx = flux(a.u[o + sx], a.u[o - sx], a.k[o + sx], a.k[o - sx]);
      const T Fy = flux(a.u[o + sy], a.u[o - sy], a.k[o + sy], a.k[o - sy]);
      const T Fz = flux(up, um, kp, km);
      res = add_rn(uc, fma_k(a.cz, Fz, fma_k(a.cy, Fy, mul_rn(a.cx, Fx))));
    } else {
      res = a.zero_boundary ? T(0) : uc;
    }
    a.out[o] = res;
    um = uc; uc = up; km = kc; kc = kp;
  }
}

template <class T>
__global__ void __launch_bounds__(512) heatk_adjoint_kernel(const __grid_constant__ HeatKArgs<T> a) {
  const int x = blockIdx.x * KX + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.nx || y >= a.ny) return;
  const int z0 = blockIdx.z * a.zc, z1 = min(a.nz, z0 + a.zc);
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
  const T h = T(0.5);
  // interior tests of this column and of its x / y neighbours' columns
  auto in1 = [](int i, int n) { return i > 0 && i < n - 1; };
  const bool xin = in1(x, nx), yin = in1(y, ny);
  const bool hxp = x + 1 < nx, hxm = x > 0, hyp = y + 1 < ny, hym = y > 0;
  const bool cxp = in1(x + 1, nx) && yin, cxm = in1(x - 1, nx) && yin;
  const bool cyp = xin && in1(y + 1, ny), cym = xin && in1(y - 1, ny);
  const bool ccol = xin && yin;
  // one axis from the neighbours' values (an absent neighbour passes the centre's values)
  auto axis = [&](bool hp, bool hm, bool inp, bool inm, T lp, T lm, T up, T um, T kp, T km, T muc, T uc, T kc, T& S,
                  T& G) {
    const T mup = hp && inp ? lp : T(0), mum = hm && inm ? lm : T(0);
    const T kfp = mul_rn(h, add_rn(kc, kp)), kfm = mul_rn(h, add_rn(kc, km));
    const T dmp = hp ? sub_rn(mup, muc) : T(0), dmm = hm ? sub_rn(mum, muc) : T(0);
    const T dup = sub_rn(up, uc), dum = sub_rn(um, uc);
    S = fma_k(kfm, dmm, mul_rn(kfp, dmp));
    G = fma_k(dum, -dmm, mul_rn(dup, -dmp));
  };
  size_t o = (size_t)x + sy * y + sz * z0;
  // z windows of lam, u, k at z-1, z, z+1
  T lc = a.lam[o], uc = a.u[o], kc = a.k[o];
  T lm = z0 > 0 ? a.lam[o - sz] : lc, um = z0 > 0 ? a.u[o - sz] : uc, km = z0 > 0 ? a.k[o - sz] : kc;
  for (int z = z0; z < z1; ++z, o += sz) {
    const bool hzp = z + 1 < nz, hzm = z > 0;
    const T lp = hzp ? a.lam[o + sz] : lc, up = hzp ? a.u[o + sz] : uc, kp = hzp ? a.k[o + sz] : kc;
    const bool zin = in1(z, nz);
    const bool in_c = ccol && zin;
    const T muc = in_c ? lc : T(0);
    const size_t ox = hxp ? o + 1 : o, oxm = hxm ? o - 1 : o, oy = hyp ? o + sy : o, oym = hym ? o - sy : o;
    T Sx, Gx, Sy, Gy, Sz, Gz;
    axis(hxp, hxm, cxp && zin, cxm && zin, a.lam[ox], a.lam[oxm], a.u[ox], a.u[oxm], a.k[ox], a.k[oxm], muc, uc, kc,
         Sx, Gx);
    axis(hyp, hym, cyp && zin, cym && zin, a.lam[oy], a.lam[oym], a.u[oy], a.u[oym], a.k[oy], a.k[oym], muc, uc, kc,
         Sy, Gy);
    axis(hzp, hzm, ccol && in1(z + 1, nz), ccol && in1(z - 1, nz), lp, lm, up, um, kp, km, muc, uc, kc, Sz, Gz);
    const T keep = (in_c || !a.zero_boundary) ? lc : T(0);
    a.out[o] = add_rn(keep, fma_k(a.cz, Sz, fma_k(a.cy, Sy, mul_rn(a.cx, Sx))));
    a.grad[o] = fma_k(h, fma_k(a.cz, Gz, fma_k(a.cy, Gy, mul_rn(a.cx, Gx))), a.grad[o]);
    lm = lc; lc = lp; um = uc; uc = up; km = kc; kc = kp;
  }
}

// ------------------------------------------------------------ vector kernels (16-byte rows)
// The same per-node arithmetic as the kernels above (so the same bits), with each thread owning
// VX = 16 / sizeof(T) consecutive nodes of a row: one 16-byte load per field and row instead of
// one per node, the nodes' x neighbours from the thread's own vector plus one scalar per side.
// Used when nx is a multiple of VX and every array is 16-byte aligned.
template <class T> struct V16;
template <> struct V16<float> { using type = float4; static constexpr int N = 4; };
template <> struct V16<double> { using type = double2; static constexpr int N = 2; };
constexpr int KXV = 16;  // threads per block row
// FP32 adjoint rows in 8-byte vectors (two nodes per thread): half the registers of 16-byte
// vectors (56 instead of 101), so twice the resident warps to cover the latency of its seven
// input streams (measured 11% faster at 192^3)
constexpr int kAdjVxF32 = 2;

// vector of N elements of T in one load / store (N * sizeof(T) = 8 or 16 bytes)
template <class T, int N> struct VecN;
template <> struct VecN<float, 4> { using type = float4; };
template <> struct VecN<float, 2> { using type = float2; };
template <> struct VecN<double, 2> { using type = double2; };
template <class T, int N>
__device__ __forceinline__ void ldvn(const T* p, T (&v)[N]) {
  const typename VecN<T, N>::type w = *reinterpret_cast<const typename VecN<T, N>::type*>(p);
#pragma unroll
  for (int e = 0; e < N; ++e) v[e] = reinterpret_cast<const T*>(&w)[e];
}
template <class T, int N>
__device__ __forceinline__ void stvn(T* p, const T (&v)[N]) {
  typename VecN<T, N>::type w;
#pragma unroll
  for (int e = 0; e < N; ++e) reinterpret_cast<T*>(&w)[e] = v[e];
  *reinterpret_cast<typename VecN<T, N>::type*>(p) = w;
}

template <class T>
__device__ __forceinline__ void ldv(const T* p, T (&v)[V16<T>::N]) {
  const typename V16<T>::type w = *reinterpret_cast<const typename V16<T>::type*>(p);
#pragma unroll
  for (int e = 0; e < V16<T>::N; ++e) v[e] = reinterpret_cast<const T*>(&w)[e];
}
template <class T>
__device__ __forceinline__ void stv(T* p, const T (&v)[V16<T>::N]) {
  typename V16<T>::type w;
#pragma unroll
  for (int e = 0; e < V16<T>::N; ++e) reinterpret_cast<T*>(&w)[e] = v[e];
  *reinterpret_cast<typename V16<T>::type*>(p) = w;
}

template <class T>
__global__ void __launch_bounds__(256) heatk_step_vec_kernel(const __grid_constant__ HeatKArgs<T> a) {
  constexpr int VX = V16<T>::N;
  const int xb = (blockIdx.x * KXV + threadIdx.x) * VX, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (xb >= a.nx || y >= a.ny) return;
  const int z0 = blockIdx.z * a.zc, z1 = min(a.nz, z0 + a.zc);
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
  const T h = T(0.5);
  const bool yin = y > 0 && y < ny - 1;
  const bool hl = xb > 0, hr = xb + VX < nx;
  size_t o = (size_t)xb + sy * y + sz * z0;
  T uc[VX], kc[VX], um[VX], km[VX];
  ldv(a.u + o, uc);
  ldv(a.k + o, kc);
  if (z0 > 0) { ldv(a.u + o - sz, um); ldv(a.k + o - sz, km); }
  else {
#pragma unroll
    for (int e = 0; e < VX; ++e) { um[e] = uc[e]; km[e] = kc[e]; }
  }
  for (int z = z0; z < z1; ++z, o += sz) {
    T up[VX], kp[VX];
    if (z + 1 < nz) { ldv(a.u + o + sz, up); ldv(a.k + o + sz, kp); }
    else {
#pragma unroll
      for (int e = 0; e < VX; ++e) { up[e] = uc[e]; kp[e] = kc[e]; }
    }
    T res[VX];
    const bool zin = z > 0 && z < nz - 1;
    if (yin && zin) {
      T uyp[VX], uym[VX], kyp[VX], kym[VX];
      ldv(a.u + o + sy, uyp); ldv(a.u + o - sy, uym); ldv(a.k + o + sy, kyp); ldv(a.k + o - sy, kym);
      const T ul = hl ? a.u[o - 1] : T(0), kl = hl ? a.k[o - 1] : T(0);
      const T ur = hr ? a.u[o + VX] : T(0), kr = hr ? a.k[o + VX] : T(0);
#pragma unroll
      for (int e = 0; e < VX; ++e) {
        const int x = xb + e;
        if (x > 0 && x < nx - 1) {
          const T c = uc[e], kce = kc[e];
          auto flux = [&](T u_p, T u_m, T k_p, T k_m) {
            const T fp = mul_rn(h, add_rn(kce, k_p)), fm = mul_rn(h, add_rn(kce, k_m));
            return fma_k(fp, sub_rn(u_p, c), -mul_rn(fm, sub_rn(c, u_m)));
          };
          const T uxp = e + 1 < VX ? uc[e + 1 < VX ? e + 1 : 0] : ur, kxp = e + 1 < VX ? kc[e + 1 < VX ? e + 1 : 0] : kr;
          const T uxm = e > 0 ? uc[e > 0 ? e - 1 : 0] : ul, kxm = e > 0 ? kc[e > 0 ? e - 1 : 0] : kl;
          const T Fx = flux(uxp, uxm, kxp, kxm);
          const T Fy = flux(uyp[e], uym[e], kyp[e], kym[e]);
          const T Fz = flux(up[e], um[e], kp[e], km[e]);
          res[e] = add_rn(c, fma_k(a.cz, Fz, fma_k(a.cy, Fy, mul_rn(a.cx, Fx))));
        } else {
          res[e] = a.zero_boundary ? T(0) : uc[e];
        }
      }
    } else {
#pragma unroll
      for (int e = 0; e < VX; ++e) res[e] = a.zero_boundary ? T(0) : uc[e];
    }
    stv(a.out + o, res);
#pragma unroll
    for (int e = 0; e < VX; ++e) { um[e] = uc[e]; uc[e] = up[e]; km[e] = kc[e]; kc[e] = kp[e]; }
  }
}

template <class T, int VXN = V16<T>::N>
__global__ void __launch_bounds__(256) heatk_adjoint_vec_kernel(const __grid_constant__ HeatKArgs<T> a) {
  constexpr int VX = VXN;
  const int xb = (blockIdx.x * blockDim.x + threadIdx.x) * VX, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (xb >= a.nx || y >= a.ny) return;
  const int z0 = blockIdx.z * a.zc, z1 = min(a.nz, z0 + a.zc);
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
  const T h = T(0.5);
  auto in1 = [](int i, int n) { return i > 0 && i < n - 1; };
  const bool yin = in1(y, ny), hyp = y + 1 < ny, hym = y > 0;
  const bool hl = xb > 0, hr = xb + VX < nx;
  auto axis = [&](bool hp, bool hm, bool inp, bool inm, T lp, T lm, T up, T um, T kp, T km, T muc, T uc, T kc, T& S,
                  T& G) {
    const T mup = hp && inp ? lp : T(0), mum = hm && inm ? lm : T(0);
    const T kfp = mul_rn(h, add_rn(kc, kp)), kfm = mul_rn(h, add_rn(kc, km));
    const T dmp = hp ? sub_rn(mup, muc) : T(0), dmm = hm ? sub_rn(mum, muc) : T(0);
    const T dup = sub_rn(up, uc), dum = sub_rn(um, uc);
    S = fma_k(kfm, dmm, mul_rn(kfp, dmp));
    G = fma_k(dum, -dmm, mul_rn(dup, -dmp));
  };
  size_t o = (size_t)xb + sy * y + sz * z0;
  T lc[VX], uc[VX], kc[VX], lm[VX], um[VX], km[VX];
  ldvn<T, VX>(a.lam + o, lc); ldvn<T, VX>(a.u + o, uc); ldvn<T, VX>(a.k + o, kc);
  if (z0 > 0) { ldvn<T, VX>(a.lam + o - sz, lm); ldvn<T, VX>(a.u + o - sz, um); ldvn<T, VX>(a.k + o - sz, km); }
  else {
#pragma unroll
    for (int e = 0; e < VX; ++e) { lm[e] = lc[e]; um[e] = uc[e]; km[e] = kc[e]; }
  }
  for (int z = z0; z < z1; ++z, o += sz) {
    const bool hzp = z + 1 < nz, hzm = z > 0;
    T lp[VX], up[VX], kp[VX];
    if (hzp) { ldvn<T, VX>(a.lam + o + sz, lp); ldvn<T, VX>(a.u + o + sz, up); ldvn<T, VX>(a.k + o + sz, kp); }
    else {
#pragma unroll
      for (int e = 0; e < VX; ++e) { lp[e] = lc[e]; up[e] = uc[e]; kp[e] = kc[e]; }
    }
    // y neighbours (an absent one passes the centre's values, as in the scalar kernel)
    T lyp[VX], uyp[VX], kyp[VX], lym[VX], uym[VX], kym[VX];
    if (hyp) { ldvn<T, VX>(a.lam + o + sy, lyp); ldvn<T, VX>(a.u + o + sy, uyp); ldvn<T, VX>(a.k + o + sy, kyp); }
    else {
#pragma unroll
      for (int e = 0; e < VX; ++e) { lyp[e] = lc[e]; uyp[e] = uc[e]; kyp[e] = kc[e]; }
    }
    if (hym) { ldvn<T, VX>(a.lam + o - sy, lym); ldvn<T, VX>(a.u + o - sy, uym); ldvn<T, VX>(a.k + o - sy, kym); }
    else {
#pragma unroll
      for (int e = 0; e < VX; ++e) { lym[e] = lc[e]; uym[e] = uc[e]; kym[e] = kc[e]; }
    }
    const T ll = hl ? a.lam[o - 1] : T(0), ul = hl ? a.u[o - 1] : T(0), kl = hl ? a.k[o - 1] : T(0);
    const T lr = hr ? a.lam[o + VX] : T(0), ur = hr ? a.u[o + VX] : T(0), kr = hr ? a.k[o + VX] : T(0);
    T g[VX], out[VX];
    ldvn<T, VX>(a.grad + o, g);
    const bool zin = in1(z, nz), zinp = in1(z + 1, nz), zinm = in1(z - 1, nz);
#pragma unroll
    for (int e = 0; e < VX; ++e) {
      const int x = xb + e;
      const bool xin = in1(x, nx), hxp = x + 1 < nx, hxm = x > 0;
      const bool ccol = xin && yin;
      const bool in_c = ccol && zin;
      const T muc = in_c ? lc[e] : T(0);
      // x neighbours of node e: inside the vector, or the scalars past its ends
      const T lxp = hxp ? (e + 1 < VX ? lc[e + 1 < VX ? e + 1 : 0] : lr) : lc[e];
      const T uxp = hxp ? (e + 1 < VX ? uc[e + 1 < VX ? e + 1 : 0] : ur) : uc[e];
      const T kxp = hxp ? (e + 1 < VX ? kc[e + 1 < VX ? e + 1 : 0] : kr) : kc[e];
      const T lxm = hxm ? (e > 0 ? lc[e > 0 ? e - 1 : 0] : ll) : lc[e];
      const T uxm = hxm ? (e > 0 ? uc[e > 0 ? e - 1 : 0] : ul) : uc[e];
      const T kxm = hxm ? (e > 0 ? kc[e > 0 ? e - 1 : 0] : kl) : kc[e];
      T Sx, Gx, Sy, Gy, Sz, Gz;
      axis(hxp, hxm, in1(x + 1, nx) && yin && zin, in1(x - 1, nx) && yin && zin, lxp, lxm, uxp, uxm, kxp, kxm, muc,
           uc[e], kc[e], Sx, Gx);
      axis(hyp, hym, xin && in1(y + 1, ny) && zin, xin && in1(y - 1, ny) && zin, lyp[e], lym[e], uyp[e], uym[e],
           kyp[e], kym[e], muc, uc[e], kc[e], Sy, Gy);
      axis(hzp, hzm, ccol && zinp, ccol && zinm, lp[e], lm[e], up[e], um[e], kp[e], km[e], muc, uc[e], kc[e], Sz, Gz);
      const T keep = (in_c || !a.zero_boundary) ? lc[e] : T(0);
      out[e] = add_rn(keep, fma_k(a.cz, Sz, fma_k(a.cy, Sy, mul_rn(a.cx, Sx))));
      g[e] = fma_k(h, fma_k(a.cz, Gz, fma_k(a.cy, Gy, mul_rn(a.cx, Gx))), g[e]);
    }
    stvn<T, VX>(a.out + o, out);
    stvn<T, VX>(a.grad + o, g);
#pragma unroll
    for (int e = 0; e < VX; ++e) {
      lm[e] = lc[e]; lc[e] = lp[e]; um[e] = uc[e]; uc[e] = up[e]; km[e] = kc[e]; kc[e] = kp[e];
    }
  }
}

adv_status heatk_validate(const adv_heatk_desc* d) {
  if (!d) return set_error(ADV_ERR_INVALID_ARG, "heatk: null descriptor");
  if (d->dtype != ADV_F32 && d->dtype != ADV_F64) return set_error(ADV_ERR_INVALID_ARG, "heatk: bad dtype");
  if (d->nx < 1 || d->ny < 1 || d->nz < 1) return set_error(ADV_ERR_INVALID_ARG, "heatk: empty grid");
  if ((int64_t)d->nx * d->ny * d->nz > ((int64_t)1 << 40) || d->nx > (1 << 30) || d->ny > (1 << 30) ||
      d->nz > (1 << 30))
    return set_error(ADV_ERR_INVALID_ARG, "heatk: grid too large");
  return ADV_OK;
}

template <class T>
HeatKArgs<T> make_args(const adv_heatk_desc& d, const void* k, const void* u, const void* lam, void* out, void* grad) {
  HeatKArgs<T> a;
  a.k = static_cast<const T*>(k);
  a.u = static_cast<const T*>(u);
  a.lam = static_cast<const T*>(lam);
  a.out = static_cast<T*>(out);
  a.grad = static_cast<T*>(grad);
  a.nx = d.nx; a.ny = d.ny; a.nz = d.nz;
  a.zero_boundary = d.zero_boundary;
  a.cx = (T)d.cx; a.cy = (T)d.cy; a.cz = (T)d.cz;
  return a;
}

// The vector kernels need whole 16-byte vectors per row and 16-byte aligned arrays.
bool vec_ok(const adv_heatk_desc& d, std::initializer_list<const void*> ptrs) {
  const int vx = d.dtype == ADV_F32 ? 4 : 2;
  if (d.nx % vx != 0) return false;
  for (const void* p : ptrs)
    if ((uintptr_t)p % 16 != 0) return false;
  return true;
}

// Block height and z planes per CTA: the autotuner's choice for this problem, else 8 and 16.
void heatk_shape(const adv_heatk_desc& d, int kind, int* ky, int* zc) {
  const TuneParams tp = tune_lookup(kind, d.dtype, d.nx, d.ny, d.nz);
  *ky = tp.set ? tp.a : 8;
  *zc = tp.set ? tp.b : 16;
}

adv_status heatk_step_launch(const adv_heatk_desc& d, const void* k, const void* u_in, void* u_out, cudaStream_t s) {
  int ky, zc;
  heatk_shape(d, TUNE_HEATK_STEP, &ky, &zc);
  const int vx = d.dtype == ADV_F32 ? 4 : 2;
  const bool vec = vec_ok(d, {k, u_in, u_out});
  const int bx = vec ? KXV : KX, xs = vec ? KXV * vx : KX;
  const dim3 grid((unsigned)((d.nx + xs - 1) / xs), (unsigned)((d.ny + ky - 1) / ky), (unsigned)((d.nz + zc - 1) / zc));
  if (d.dtype == ADV_F32) {
    HeatKArgs<float> a = make_args<float>(d, k, u_in, nullptr, u_out, nullptr);
    a.zc = zc;
    if (vec) heatk_step_vec_kernel<float><<<grid, dim3(bx, ky), 0, s>>>(a);
    else heatk_step_kernel<float><<<grid, dim3(bx, ky), 0, s>>>(a);
  } else {
    HeatKArgs<double> a = make_args<double>(d, k, u_in, nullptr, u_out, nullptr);
    a.zc = zc;
    if (vec) heatk_step_vec_kernel<double><<<grid, dim3(bx, ky), 0, s>>>(a);
    else heatk_step_kernel<double><<<grid, dim3(bx, ky), 0, s>>>(a);
  }
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}

adv_status heatk_adjoint_launch(const adv_heatk_desc& d, const void* k, const void* u_n, const void* lam_next,
                                void* lam_out, void* grad_k, cudaStream_t s) {
  int ky, zc;
  heatk_shape(d, TUNE_HEATK_ADJ, &ky, &zc);
  const int vx = d.dtype == ADV_F32 ? kAdjVxF32 : 2;
  const bool vec = vec_ok(d, {k, u_n, lam_next, lam_out, grad_k});
  const int bx = vec ? KXV : KX, xs = vec ? KXV * vx : KX;
  const dim3 grid((unsigned)((d.nx + xs - 1) / xs), (unsigned)((d.ny + ky - 1) / ky), (unsigned)((d.nz + zc - 1) / zc));
  if (d.dtype == ADV_F32) {
    HeatKArgs<float> a = make_args<float>(d, k, u_n, lam_next, lam_out, grad_k);
    a.zc = zc;
    if (vec) heatk_adjoint_vec_kernel<float, kAdjVxF32><<<grid, dim3(bx, ky), 0, s>>>(a);
    else heatk_adjoint_kernel<float><<<grid, dim3(bx, ky), 0, s>>>(a);
  } else {
    HeatKArgs<double> a = make_args<double>(d, k, u_n, lam_next, lam_out, grad_k);
    a.zc = zc;
    if (vec) heatk_adjoint_vec_kernel<double><<<grid, dim3(bx, ky), 0, s>>>(a);
    else heatk_adjoint_kernel<double><<<grid, dim3(bx, ky), 0, s>>>(a);
  }
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}

size_t array_bytes(const adv_heatk_desc& d) {
  const size_t n = (size_t)d.nx * d.ny * d.nz * (d.dtype == ADV_F32 ? 4 : 8);
  return (n + 255) / 256 * 256;
}

}  // namespace

// for the autotuner
adv_status heatk_validate_desc(const adv_heatk_desc* d) { return heatk_validate(d); }
adv_status heatk_step_run(const adv_heatk_desc& d, const void* k, const void* u_in, void* u_out, cudaStream_t s) {
  return heatk_step_launch(d, k, u_in, u_out, s);
}
adv_status heatk_adjoint_run(const adv_heatk_desc& d, const void* k, const void* u_n, const void* lam_next,
                             void* lam_out, void* grad_k, cudaStream_t s) {
  return heatk_adjoint_launch(d, k, u_n, lam_next, lam_out, grad_k, s);
}

}  // namespace adv

using namespace adv;

extern "C" {

adv_status adv_heatk_step(const adv_heatk_desc* d, const void* k, const void* u_in, void* u_out, void* stream) {
  ADV_NVTX_RANGE("adv_heatk_step");
  adv_status st = heatk_validate(d);
  if (st != ADV_OK) return st;
  if (!k || !u_in || !u_out) return set_error(ADV_ERR_INVALID_ARG, "heatk: null buffer");
  if (u_in == u_out) return set_error(ADV_ERR_INVALID_ARG, "heatk: u_in and u_out must not alias");
  return heatk_step_launch(*d, k, u_in, u_out, static_cast<cudaStream_t>(stream));
}

adv_status adv_heatk_adjoint_step(const adv_heatk_desc* d, const void* k, const void* u_n, const void* lam_next,
                                  void* lam_out, void* grad_k, void* stream) {
  ADV_NVTX_RANGE("adv_heatk_adjoint_step");
  adv_status st = heatk_validate(d);
  if (st != ADV_OK) return st;
  if (!k || !u_n || !lam_next || !lam_out || !grad_k) return set_error(ADV_ERR_INVALID_ARG, "heatk: null buffer");
  if (lam_next == lam_out) return set_error(ADV_ERR_INVALID_ARG, "heatk: lam_next and lam_out must not alias");
  return heatk_adjoint_launch(*d, k, u_n, lam_next, lam_out, grad_k, static_cast<cudaStream_t>(stream));
}

adv_status adv_heatk_checkpoint_bytes(const adv_heatk_desc* d, int64_t nsteps, int64_t interval, size_t* ckpt_bytes,
                                      size_t* work_bytes) {
  adv_status st = heatk_validate(d);
  if (st != ADV_OK) return st;
  if (nsteps < 0 || interval < 1) return set_error(ADV_ERR_INVALID_ARG, "heatk: bad nsteps/interval");
  const size_t one = array_bytes(*d);
  const int64_t m = (nsteps + interval - 1) / interval;
  if (ckpt_bytes) *ckpt_bytes = (size_t)std::max<int64_t>(m, 1) * one;
  // forward: one ping-pong array; backward: the segment's states (interval - 1 beyond the
  // checkpoint) and one adjoint ping-pong array
  if (work_bytes) *work_bytes = (size_t)std::max<int64_t>(interval, 1) * one;
  return ADV_OK;
}

adv_status adv_heatk_forward(const adv_heatk_desc* d, const void* k, void* u, int64_t nsteps, int64_t interval,
                             void* ckpt, void* work, void* stream) {
  ADV_NVTX_RANGE("adv_heatk_forward");
  adv_status st = heatk_validate(d);
  if (st != ADV_OK) return st;
  if (!k || !u || !work) return set_error(ADV_ERR_INVALID_ARG, "heatk: null buffer");
  if (nsteps < 0 || interval < 1) return set_error(ADV_ERR_INVALID_ARG, "heatk: bad nsteps/interval");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t one = array_bytes(*d);
  const size_t nb = (size_t)d->nx * d->ny * d->nz * (d->dtype == ADV_F32 ? 4 : 8);
  char* const ub = static_cast<char*>(u);
  char* const wb = static_cast<char*>(work);
  char* const cb = static_cast<char*>(ckpt);
  // A step whose result is a checkpoint writes it into its slot (only u^0 is copied), so storing
  // checkpoints costs no traffic beyond the steps themselves; with interval 1 every state is kept
  // and the backward run recomputes nothing. The last interval runs from its checkpoint through
  // work's slots (the states u^{n0+1} .. u^{nsteps-1}, where adv_heatk_backward would recompute
  // them) into u.
  const int64_t m = (nsteps + interval - 1) / interval;
  const int64_t n_last = ckpt && nsteps > 0 ? (m - 1) * interval : nsteps;
  const char* src = ub;
  if (ckpt && nsteps > 0) ADV_CUDA_TRY(cudaMemcpyAsync(cb, ub, nb, cudaMemcpyDeviceToDevice, s));
  for (int64_t n = 0; n < n_last; ++n) {
    char* dst = ckpt && (n + 1) % interval == 0 ? cb + ((n + 1) / interval) * one : (src == ub ? wb : ub);
    if ((st = heatk_step_launch(*d, k, src, dst, s)) != ADV_OK) return st;
    src = dst;
  }
  if (n_last < nsteps) {
    src = cb + (m - 1) * one;  // u^{n_last}: the copy of u^0 or the step that wrote it there
    for (int64_t n = n_last; n < nsteps; ++n) {
      char* dst = n + 1 < nsteps ? wb + (n - n_last) * one : ub;
      if ((st = heatk_step_launch(*d, k, src, dst, s)) != ADV_OK) return st;
      src = dst;
    }
  } else if (src != ub) {
    ADV_CUDA_TRY(cudaMemcpyAsync(ub, src, nb, cudaMemcpyDeviceToDevice, s));
  }
  return ADV_OK;
}

adv_status adv_heatk_backward(const adv_heatk_desc* d, const void* k, int64_t nsteps, int64_t interval,
                              const void* ckpt, void* lam, void* grad_k, void* work, int flags, void* stream) {
  ADV_NVTX_RANGE("adv_heatk_backward");
  adv_status st = heatk_validate(d);
  if (st != ADV_OK) return st;
  if (!k || !ckpt || !lam || !grad_k || !work) return set_error(ADV_ERR_INVALID_ARG, "heatk: null buffer");
  if (nsteps < 0 || interval < 1) return set_error(ADV_ERR_INVALID_ARG, "heatk: bad nsteps/interval");
  if (flags & ~ADV_HEATK_LAST_INTERVAL_IN_WORK) return set_error(ADV_ERR_INVALID_ARG, "heatk: unknown flags");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t one = array_bytes(*d);
  const size_t nb = (size_t)d->nx * d->ny * d->nz * (d->dtype == ADV_F32 ? 4 : 8);
  char* states = static_cast<char*>(work);              // u^{n0+1} .. u^{n0+interval-1}
  char* lam_b = states + (size_t)(interval - 1) * one;  // adjoint ping-pong
  char* la = static_cast<char*>(lam);
  char* lb = lam_b;
  const int64_t m = (nsteps + interval - 1) / interval;
  for (int64_t seg = m - 1; seg >= 0; --seg) {
    const int64_t n0 = seg * interval, n1 = std::min(nsteps, n0 + interval);
    const char* base = static_cast<const char*>(ckpt) + seg * one;
    auto state = [&](int64_t n) -> const char* { return n == n0 ? base : states + (n - n0 - 1) * one; };
    const bool kept = seg == m - 1 && (flags & ADV_HEATK_LAST_INTERVAL_IN_WORK);
    for (int64_t n = n0; !kept && n + 1 < n1; ++n)
      if ((st = heatk_step_launch(*d, k, state(n), states + (n - n0) * one, s)) != ADV_OK) return st;
    for (int64_t n = n1 - 1; n >= n0; --n) {
      if ((st = heatk_adjoint_launch(*d, k, state(n), la, lb, grad_k, s)) != ADV_OK) return st;
      std::swap(la, lb);
    }
  }
  if (la != static_cast<char*>(lam)) ADV_CUDA_TRY(cudaMemcpyAsync(lam, la, nb, cudaMemcpyDeviceToDevice, s));
  return ADV_OK;
}

}  // extern "C"
