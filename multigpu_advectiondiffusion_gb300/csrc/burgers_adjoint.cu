// burgers_adjoint.cu -- discrete adjoint of the periodic, local Lax-Friedrichs WENO5 / WENO5-Z
// SSP-RK3 Burgers step, and the checkpointed forward / backward runs (adv_burgers_forward,
// adv_burgers_backward, adv_burgers_adjoint_step in advdiff.h). No reference counterpart.
//
// One adjoint stage computes, for the stage input v and the incoming adjoint lam,
//   t = lam + dt J(v)^T lam,   J = dL/dv,   L_i = -sum_a (F_{i+1/2} - F_{i-1/2}) / h_a
// and combines t into the stage outputs (see below). With psi_f = (lam_{i+1} - lam_i)/h_a the
// weight of face f = i+1/2, (J^T lam)_j = sum_f psi_f dF_f/dv_j. A face's flux is
// side(f+ at i-2..i+2) + side(f- at i+3..i-1); reverse-mode differentiation of each side gives
// five partials, which land on the ten cells of the face's stencil through f+-'(v) =
// v/2 +- |v| (local LF: f+- = v (v/4 +- |v|/2)). A cell therefore collects from the faces
// i-3..i+2 of each axis, which reach cells up to 5 away, so the adjoint needs a halo of 5 for v
// and 3 for lam.
//
// Work layout (one wave of CTAs, balanced (tile, z-plane) segments as in the forward stage): a
// CTA owns 32 x 16 columns and streams the planes z-5 .. z+4 of its segment through an 8-slot
// shared ring (v and lam with a 5-cell periodic halo, cp.async). Per streamed plane p each
// thread advances its two columns' z windows and differentiates the z-face p-3+1/2, pushing the
// partials into per-column accumulators for cells p-5..p; cell p-5 is then complete in z. For
// that plane the x- and y-faces of the tile (37 x 16 and 32 x 21) are differentiated by all
// threads into shared memory (structure of arrays), each cell gathers its ten partials per axis,
// and the stage output is written. Every face is differentiated once per pass.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "adv_device.cuh"
#include "adv_internal.h"
#include "nvtx_range.h"
#include "adv_math.cuh"

namespace adv {

namespace {

struct AdjTile {
  static constexpr int BX = 32, BY = 16, NT = 256;
  static constexpr int H = 5;                  // halo of the staged region (v needs 5, lam 3)
  static constexpr int SW = BX + 2 * H;        // 42
  static constexpr int SH = BY + 2 * H;        // 26
  static constexpr int PLANE = SW * SH;        // 1092
  static constexpr int NS = 8;                 // ring slots: planes p-5 .. p+2
  static constexpr int P = 2;                  // planes prefetched ahead
  static constexpr int NFX = (BX + 5) * BY;    // x-faces i+1/2, i = -3 .. 33, per row: 592
  static constexpr int NFY = BX * (BY + 5);    // y-faces: 672
  static constexpr int NF = NFY > NFX ? NFY : NFX;
};

template <class T>
struct AdjSmem {
  static constexpr int SLOT = ((AdjTile::PLANE * (int)sizeof(T) + 127) / 128 * 128) / (int)sizeof(T);
  static constexpr size_t RING = (size_t)AdjTile::NS * 2 * SLOT * sizeof(T);  // v and lam per slot
  static constexpr size_t FPM = (size_t)2 * SLOT * sizeof(T);                 // f+ and f- of a plane
  static constexpr size_t FB = (size_t)10 * AdjTile::NF * sizeof(T);          // face partials (SoA)
  static constexpr size_t TOTAL = RING + FPM + FB;
};

template <class T>
struct AdjArgs {
  const T* v;       // stage input (forward state)
  const T* lam;     // incoming adjoint of the stage output
  const T* acc_in;  // accumulated adjoint of u^n (stages 2, 1)
  T* out;           // outgoing adjoint (lam of the previous stage, or of u^n at stage 1)
  T* acc_out;       // accumulated adjoint of u^n (stages 3, 2); may equal acc_in
  int nx, ny, nz, stage;
  int tiles_x, tiles_y;
  T dt, rdx, rdy, rdz;
};

template <class T> __device__ __forceinline__ T absv(T x) { return fabs(x); }
template <> __device__ __forceinline__ float absv<float>(float x) { return fabsf(x); }
__device__ __forceinline__ float rcp(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp(double x) { return 1.0 / x; }

// Periodic index. Inside the domain (every element of an interior tile) it is the index itself,
// without the integer division of the general case.
__device__ __forceinline__ int wrap(int i, int n) {
  if (i >= 0 && i < n) return i;
  i %= n;
  return i < 0 ? i + n : i;
}

template <class T> __device__ __forceinline__ T fplus(T u) { return u * (T(0.25) * u + T(0.5) * absv(u)); }
template <class T> __device__ __forceinline__ T fminus(T u) { return u * (T(0.25) * u - T(0.5) * absv(u)); }

// d side(a..e) / d(a..e) times ybar, for the common-denominator weights (see the header).
template <class T, bool Z>
__device__ __forceinline__ void side_rev(T a, T b, T c, T d, T e, T ybar, T& ga, T& gb, T& gc, T& gd, T& ge) {
  const T t0 = a - T(2) * b + c, t1 = b - T(2) * c + d, t2 = c - T(2) * d + e;
  const T s0 = a - T(4) * b + T(3) * c, s1 = b - d, s2 = T(3) * c - T(4) * d + e;
  const T K = T(13.0 / 3.0), E = T(4e-6);
  const T B0 = K * t0 * t0 + s0 * s0 + E, B1 = K * t1 * t1 + s1 * s1 + E, B2 = K * t2 * t2 + s2 * s2 + E;
  const T q0 = c + t0 * T(1.0 / 12.0) + s0 * T(0.25), q1 = c + t1 * T(1.0 / 12.0) - s1 * T(0.25),
          q2 = c + t2 * T(1.0 / 12.0) - s2 * T(0.25);
  T w0, w1, w2, tau = T(0);
  T Bb0, Bb1, Bb2;
  if (Z) {
    tau = absv(B0 - B2);
    const T P0 = B0 + tau, P1 = B1 + tau, P2 = B2 + tau;
    const T b12 = B1 * B2, b02 = B0 * B2, b01 = B0 * B1;
    w0 = P0 * b12;
    w1 = T(6) * P1 * b02;
    w2 = T(3) * P2 * b01;
    const T rD = rcp(w0 + w1 + w2);
    const T side = (w0 * q0 + w1 * q1 + w2 * q2) * rD;
    const T Nb = ybar * rD;
    const T wb0 = Nb * (q0 - side), wb1 = T(6) * Nb * (q1 - side), wb2 = T(3) * Nb * (q2 - side);
    const T taub = wb0 * b12 + wb1 * b02 + wb2 * b01;
    Bb0 = wb0 * b12 + wb1 * P1 * B2 + wb2 * P2 * B1;
    Bb1 = wb0 * P0 * B2 + wb1 * b02 + wb2 * P2 * B0;
    Bb2 = wb0 * P0 * B1 + wb1 * P1 * B0 + wb2 * b01;
    const T sg = B0 > B2 ? T(1) : (B0 < B2 ? T(-1) : T(0));
    Bb0 += sg * taub;
    Bb2 -= sg * taub;
    const T qb0 = Nb * w0, qb1 = Nb * w1, qb2 = Nb * w2;
    const T tb0 = T(2) * K * t0 * Bb0 + qb0 * T(1.0 / 12.0), tb1 = T(2) * K * t1 * Bb1 + qb1 * T(1.0 / 12.0),
            tb2 = T(2) * K * t2 * Bb2 + qb2 * T(1.0 / 12.0);
    const T sb0 = T(2) * s0 * Bb0 + qb0 * T(0.25), sb1 = T(2) * s1 * Bb1 - qb1 * T(0.25),
            sb2 = T(2) * s2 * Bb2 - qb2 * T(0.25);
    const T cb = qb0 + qb1 + qb2;
    ga = tb0 + sb0;
    gb = T(-2) * tb0 + tb1 - T(4) * sb0 + sb1;
    gc = tb0 - T(2) * tb1 + tb2 + T(3) * sb0 + T(3) * sb2 + cb;
    gd = tb1 - T(2) * tb2 - sb1 - T(4) * sb2;
    ge = tb2 + sb2;
  } else {
    const T p12 = B1 * B2, p02 = B0 * B2, p01 = B0 * B1;
    w0 = p12 * p12;
    w1 = T(6) * p02 * p02;
    w2 = T(3) * p01 * p01;
    const T rD = rcp(w0 + w1 + w2);
    const T side = (w0 * q0 + w1 * q1 + w2 * q2) * rD;
    const T Nb = ybar * rD;
    const T wb0 = Nb * (q0 - side), wb1 = Nb * (q1 - side), wb2 = Nb * (q2 - side);
    Bb0 = T(12) * wb1 * p02 * B2 + T(6) * wb2 * p01 * B1;
    Bb1 = T(2) * wb0 * p12 * B2 + T(6) * wb2 * p01 * B0;
    Bb2 = T(2) * wb0 * p12 * B1 + T(12) * wb1 * p02 * B0;
    const T qb0 = Nb * w0, qb1 = Nb * w1, qb2 = Nb * w2;
    const T tb0 = T(2) * K * t0 * Bb0 + qb0 * T(1.0 / 12.0), tb1 = T(2) * K * t1 * Bb1 + qb1 * T(1.0 / 12.0),
            tb2 = T(2) * K * t2 * Bb2 + qb2 * T(1.0 / 12.0);
    const T sb0 = T(2) * s0 * Bb0 + qb0 * T(0.25), sb1 = T(2) * s1 * Bb1 - qb1 * T(0.25),
            sb2 = T(2) * s2 * Bb2 - qb2 * T(0.25);
    const T cb = qb0 + qb1 + qb2;
    ga = tb0 + sb0;
    gb = T(-2) * tb0 + tb1 - T(4) * sb0 + sb1;
    gc = tb0 - T(2) * tb1 + tb2 + T(3) * sb0 + T(3) * sb2 + cb;
    gd = tb1 - T(2) * tb2 - sb1 - T(4) * sb2;
    ge = tb2 + sb2;
  }
}

// FP32: the two sides of one face (f+ in lane x, f- in lane y) differentiated together with
// Blackwell's paired FP32 instructions (FFMA2 / FADD2 / FMUL2), the same algebra as side_rev.
__device__ __forceinline__ float2 c2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 ad2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sb2(float2 a, float2 b) { return __ffma2_rn(b, c2(-1.f), a); }
__device__ __forceinline__ float2 ml2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fm2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

template <bool Z>
__device__ __forceinline__ void side_rev2(float2 a, float2 b, float2 c, float2 d, float2 e, float2 ybar, float2 (&g)[5]) {
  const float2 m2 = c2(-2.f), m4 = c2(-4.f), p3 = c2(3.f), r12 = c2(1.f / 12.f), qt = c2(0.25f);
  const float2 t0 = ad2(fm2(m2, b, a), c), t1 = ad2(fm2(m2, c, b), d), t2 = ad2(fm2(m2, d, c), e);
  const float2 s0 = fm2(p3, c, fm2(m4, b, a)), s1 = sb2(b, d), s2 = fm2(p3, c, fm2(m4, d, e));
  const float2 K = c2(13.f / 3.f), E = c2(4e-6f);
  const float2 B0 = fm2(ml2(K, t0), t0, fm2(s0, s0, E)), B1 = fm2(ml2(K, t1), t1, fm2(s1, s1, E)),
               B2 = fm2(ml2(K, t2), t2, fm2(s2, s2, E));
  const float2 q0 = fm2(qt, s0, fm2(r12, t0, c)), q1 = fm2(c2(-0.25f), s1, fm2(r12, t1, c)),
               q2 = fm2(c2(-0.25f), s2, fm2(r12, t2, c));
  float2 w0, w1, w2, Bb0, Bb1, Bb2;
  if (Z) {
    const float2 d02 = sb2(B0, B2);
    const float2 tau = make_float2(fabsf(d02.x), fabsf(d02.y));
    const float2 sg = make_float2(d02.x > 0.f ? 1.f : (d02.x < 0.f ? -1.f : 0.f),
                                  d02.y > 0.f ? 1.f : (d02.y < 0.f ? -1.f : 0.f));
    const float2 P0 = ad2(B0, tau), P1 = ad2(B1, tau), P2 = ad2(B2, tau);
    const float2 b12 = ml2(B1, B2), b02 = ml2(B0, B2), b01 = ml2(B0, B1);
    w0 = ml2(P0, b12);
    w1 = ml2(ml2(c2(6.f), P1), b02);
    w2 = ml2(ml2(p3, P2), b01);
    const float2 den = ad2(ad2(w0, w1), w2);
    const float2 rD = make_float2(__frcp_rn(den.x), __frcp_rn(den.y));
    const float2 side = ml2(fm2(w2, q2, fm2(w1, q1, ml2(w0, q0))), rD);
    const float2 Nb = ml2(ybar, rD);
    const float2 wb0 = ml2(Nb, sb2(q0, side)), wb1 = ml2(ml2(c2(6.f), Nb), sb2(q1, side)),
                 wb2 = ml2(ml2(p3, Nb), sb2(q2, side));
    const float2 taub = fm2(wb2, b01, fm2(wb1, b02, ml2(wb0, b12)));
    Bb0 = fm2(wb2, ml2(P2, B1), fm2(wb1, ml2(P1, B2), ml2(wb0, b12)));
    Bb1 = fm2(wb2, ml2(P2, B0), fm2(wb1, b02, ml2(wb0, ml2(P0, B2))));
    Bb2 = fm2(wb2, b01, fm2(wb1, ml2(P1, B0), ml2(wb0, ml2(P0, B1))));
    Bb0 = fm2(sg, taub, Bb0);
    Bb2 = fm2(make_float2(-sg.x, -sg.y), taub, Bb2);
    const float2 qb0 = ml2(Nb, w0), qb1 = ml2(Nb, w1), qb2 = ml2(Nb, w2);
    const float2 K2 = c2(26.f / 3.f);
    const float2 tb0 = fm2(ml2(K2, t0), Bb0, ml2(qb0, r12)), tb1 = fm2(ml2(K2, t1), Bb1, ml2(qb1, r12)),
                 tb2 = fm2(ml2(K2, t2), Bb2, ml2(qb2, r12));
    const float2 sv0 = fm2(ml2(c2(2.f), s0), Bb0, ml2(qb0, qt)), sv1 = fm2(ml2(c2(2.f), s1), Bb1, ml2(qb1, c2(-0.25f))),
                 sv2 = fm2(ml2(c2(2.f), s2), Bb2, ml2(qb2, c2(-0.25f)));
    const float2 cb = ad2(ad2(qb0, qb1), qb2);
    g[0] = ad2(tb0, sv0);
    g[1] = ad2(fm2(m2, tb0, tb1), fm2(m4, sv0, sv1));
    g[2] = ad2(fm2(m2, tb1, ad2(tb0, tb2)), fm2(p3, ad2(sv0, sv2), cb));
    g[3] = fm2(m4, sv2, sb2(fm2(m2, tb2, tb1), sv1));
    g[4] = ad2(tb2, sv2);
  } else {
    const float2 p12 = ml2(B1, B2), p02 = ml2(B0, B2), p01 = ml2(B0, B1);
    w0 = ml2(p12, p12);
    w1 = ml2(ml2(c2(6.f), p02), p02);
    w2 = ml2(ml2(p3, p01), p01);
    const float2 den = ad2(ad2(w0, w1), w2);
    const float2 rD = make_float2(__frcp_rn(den.x), __frcp_rn(den.y));
    const float2 side = ml2(fm2(w2, q2, fm2(w1, q1, ml2(w0, q0))), rD);
    const float2 Nb = ml2(ybar, rD);
    const float2 wb0 = ml2(Nb, sb2(q0, side)), wb1 = ml2(Nb, sb2(q1, side)), wb2 = ml2(Nb, sb2(q2, side));
    Bb0 = fm2(ml2(c2(12.f), wb1), ml2(p02, B2), ml2(ml2(c2(6.f), wb2), ml2(p01, B1)));
    Bb1 = fm2(ml2(c2(2.f), wb0), ml2(p12, B2), ml2(ml2(c2(6.f), wb2), ml2(p01, B0)));
    Bb2 = fm2(ml2(c2(2.f), wb0), ml2(p12, B1), ml2(ml2(c2(12.f), wb1), ml2(p02, B0)));
    const float2 qb0 = ml2(Nb, w0), qb1 = ml2(Nb, w1), qb2 = ml2(Nb, w2);
    const float2 K2 = c2(26.f / 3.f);
    const float2 tb0 = fm2(ml2(K2, t0), Bb0, ml2(qb0, r12)), tb1 = fm2(ml2(K2, t1), Bb1, ml2(qb1, r12)),
                 tb2 = fm2(ml2(K2, t2), Bb2, ml2(qb2, r12));
    const float2 sv0 = fm2(ml2(c2(2.f), s0), Bb0, ml2(qb0, qt)), sv1 = fm2(ml2(c2(2.f), s1), Bb1, ml2(qb1, c2(-0.25f))),
                 sv2 = fm2(ml2(c2(2.f), s2), Bb2, ml2(qb2, c2(-0.25f)));
    const float2 cb = ad2(ad2(qb0, qb1), qb2);
    g[0] = ad2(tb0, sv0);
    g[1] = ad2(fm2(m2, tb0, tb1), fm2(m4, sv0, sv1));
    g[2] = ad2(fm2(m2, tb1, ad2(tb0, tb2)), fm2(p3, ad2(sv0, sv2), cb));
    g[3] = fm2(m4, sv2, sb2(fm2(m2, tb2, tb1), sv1));
    g[4] = ad2(tb2, sv2);
  }
}

// Both sides of one face: gp[k] = d side(pv) / d pv[k] * psi and gm[k] = d side(mv) / d mv[k] * psi.
template <class T, bool Z>
__device__ __forceinline__ void sides_rev(const T (&pv)[5], const T (&mv)[5], T psi, T (&gp)[5], T (&gm)[5]) {
  if constexpr (sizeof(T) == 4) {
    float2 g[5];
    side_rev2<Z>(make_float2(pv[0], mv[0]), make_float2(pv[1], mv[1]), make_float2(pv[2], mv[2]),
                 make_float2(pv[3], mv[3]), make_float2(pv[4], mv[4]), c2(psi), g);
#pragma unroll
    for (int k = 0; k < 5; ++k) { gp[k] = g[k].x; gm[k] = g[k].y; }
  } else {
    side_rev<T, Z>(pv[0], pv[1], pv[2], pv[3], pv[4], psi, gp[0], gp[1], gp[2], gp[3], gp[4]);
    side_rev<T, Z>(mv[0], mv[1], mv[2], mv[3], mv[4], psi, gm[0], gm[1], gm[2], gm[3], gm[4]);
  }
}

// Partials of one face from the six cells v[0..5] = v at i-2 .. i+3 (split inside) and its
// weight psi: P[k] for f+ at i-2+k, M[k] for f- at i-1+k.
template <class T, bool Z>
__device__ __forceinline__ void face_rev(const T* v, T psi, T* P, T* M) {
  const T pv[5] = {fplus(v[0]), fplus(v[1]), fplus(v[2]), fplus(v[3]), fplus(v[4])};
  const T mv[5] = {fminus(v[5]), fminus(v[4]), fminus(v[3]), fminus(v[2]), fminus(v[1])};
  T gp[5], gm[5];
  sides_rev<T, Z>(pv, mv, psi, gp, gm);
#pragma unroll
  for (int k = 0; k < 5; ++k) { P[k] = gp[k]; M[4 - k] = gm[k]; }
}

template <class T, bool Z>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 2 : 1) burgers_adjoint_kernel(const __grid_constant__ AdjArgs<T> a) {
  using TL = AdjTile;
  using SM = AdjSmem<T>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* ring = reinterpret_cast<T*>(smem_raw);  // slot s: v at ring + 2 s SLOT, lam at + SLOT
  T* fpS = reinterpret_cast<T*>(smem_raw + SM::RING);
  T* fmS = fpS + SM::SLOT;
  T* FB = reinterpret_cast<T*>(smem_raw + SM::RING + SM::FPM);  // [10][NF]: P0..P4, M0..M4

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const size_t sxy = (size_t)nx * ny;
  const int64_t total = (int64_t)a.tiles_x * a.tiles_y * nz;
  const int64_t seg_a = total * blockIdx.x / gridDim.x, seg_b = total * (blockIdx.x + 1) / gridDim.x;
  const int cx = lane, cy0 = warp, cy1 = warp + 8;

  for (int64_t pos = seg_a; pos < seg_b;) {
    const int64_t tile = pos / nz;
    const int zs = (int)(pos - tile * nz);
    const int ze = (int)min((int64_t)nz, zs + (seg_b - pos));
    pos += ze - zs;
    const int x0 = (int)(tile % a.tiles_x) * TL::BX, y0 = (int)(tile / a.tiles_x) * TL::BY;
    const int Q = (ze - zs) + 10;  // planes zs-5 .. ze+4
    int s_issue = 0;
    auto issue = [&](int q) {
      T* dv = ring + (size_t)(2 * s_issue) * SM::SLOT;
      T* dl = dv + SM::SLOT;
      const int z = wrap(zs - 5 + q, nz);
      const size_t zo = (size_t)z * sxy;
      for (int e = tid; e < TL::PLANE; e += TL::NT) {
        const int r = e / TL::SW, c = e - r * TL::SW;
        const size_t o = zo + (size_t)wrap(y0 - TL::H + r, ny) * nx + wrap(x0 - TL::H + c, nx);
        cp_async_zfill<sizeof(T)>(dv + e, a.v + o, true);
        cp_async_zfill<sizeof(T)>(dl + e, a.lam + o, true);
      }
      cp_async_commit();
      s_issue = s_issue + 1 == TL::NS ? 0 : s_issue + 1;
    };
    auto slot_of = [&](int q) { return q % TL::NS; };
    for (int q = 0; q <= TL::P; ++q) issue(q);  // Q >= 11 > P

    T vw[2][6];                 // v at p-5 .. p per column
    T accP[2][6], accM[2][6];   // partial sums for cells p-5 .. p
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
      for (int k = 0; k < 6; ++k) { vw[c][k] = T(0); accP[c][k] = T(0); accM[c][k] = T(0); }

    for (int q = 0; q < Q; ++q) {
      cp_async_wait<TL::P>();
      __syncthreads();  // plane q visible
      const T* vq = ring + (size_t)(2 * slot_of(q)) * SM::SLOT;
      // ---- z: windows and the face p-3+1/2 (p = plane q)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int cy = c ? cy1 : cy0;
        const int ci = (cy + TL::H) * TL::SW + TL::H + cx;
#pragma unroll
        for (int k = 0; k < 5; ++k) vw[c][k] = vw[c][k + 1];
        vw[c][5] = vq[ci];
        if (q >= 5) {
          const T* l3 = ring + (size_t)(2 * slot_of(q - 3)) * SM::SLOT + SM::SLOT;
          const T* l2 = ring + (size_t)(2 * slot_of(q - 2)) * SM::SLOT + SM::SLOT;
          const T psi = a.rdz * (l2[ci] - l3[ci]);
          T P[5], M[5];
          face_rev<T, Z>(vw[c], psi, P, M);
#pragma unroll
          for (int k = 0; k < 5; ++k) { accP[c][k] += P[k]; accM[c][k + 1] += M[k]; }
        }
      }
      if (q >= 10) {
        // ---- output plane o = plane q-5: its x- and y-faces
        const int so = slot_of(q - 5);
        const T* vo = ring + (size_t)(2 * so) * SM::SLOT;
        const T* lo = vo + SM::SLOT;
        for (int e = tid; e < TL::PLANE; e += TL::NT) {
          const T u = vo[e];
          fpS[e] = fplus(u);
          fmS[e] = fminus(u);
        }
        __syncthreads();
        T gP[2], gM[2];
        // x-faces: face f = r * 37 + (i + 3), i = -3 .. 33, of row r
        for (int f = tid; f < TL::NFX; f += TL::NT) {
          const int r = f / (TL::BX + 5), i = f - r * (TL::BX + 5) - 3;
          const int b = (r + TL::H) * TL::SW + TL::H + i;  // region index of cell i
          const T psi = a.rdx * (lo[b + 1] - lo[b]);
          const T pv[5] = {fpS[b - 2], fpS[b - 1], fpS[b], fpS[b + 1], fpS[b + 2]};
          const T mv[5] = {fmS[b + 3], fmS[b + 2], fmS[b + 1], fmS[b], fmS[b - 1]};
          T gp[5], gm[5];
          sides_rev<T, Z>(pv, mv, psi, gp, gm);
#pragma unroll
          for (int k = 0; k < 5; ++k) {
            FB[k * TL::NF + f] = gp[k];
            FB[(5 + k) * TL::NF + f] = gm[4 - k];
          }
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int cy = c ? cy1 : cy0;
          const int fr = cy * (TL::BX + 5) + 3;  // face index of i = 0 in row cy
          T sp = T(0), sm = T(0);
#pragma unroll
          for (int d = -2; d <= 2; ++d) sp += FB[(2 - d) * TL::NF + fr + cx + d];       // faces cx-2 .. cx+2
#pragma unroll
          for (int d = -3; d <= 1; ++d) sm += FB[(5 + 1 - d) * TL::NF + fr + cx + d];   // faces cx-3 .. cx+1
          gP[c] = sp;
          gM[c] = sm;
        }
        __syncthreads();
        // y-faces: face f = (j + 3) * 32 + col, j = -3 .. 17
        for (int f = tid; f < TL::NFY; f += TL::NT) {
          const int jj = f / TL::BX, col = f - jj * TL::BX, j = jj - 3;
          const int b = (j + TL::H) * TL::SW + TL::H + col;
          constexpr int W = TL::SW;
          const T psi = a.rdy * (lo[b + W] - lo[b]);
          const T pv[5] = {fpS[b - 2 * W], fpS[b - W], fpS[b], fpS[b + W], fpS[b + 2 * W]};
          const T mv[5] = {fmS[b + 3 * W], fmS[b + 2 * W], fmS[b + W], fmS[b], fmS[b - W]};
          T gp[5], gm[5];
          sides_rev<T, Z>(pv, mv, psi, gp, gm);
#pragma unroll
          for (int k = 0; k < 5; ++k) {
            FB[k * TL::NF + f] = gp[k];
            FB[(5 + k) * TL::NF + f] = gm[4 - k];
          }
        }
        __syncthreads();
        const int ko = wrap(zs - 5 + q - 5, nz);
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int cy = c ? cy1 : cy0;
          T sp = T(0), sm = T(0);
#pragma unroll
          for (int d = -2; d <= 2; ++d) sp += FB[(2 - d) * TL::NF + (cy + d + 3) * TL::BX + cx];
#pragma unroll
          for (int d = -3; d <= 1; ++d) sm += FB[(5 + 1 - d) * TL::NF + (cy + d + 3) * TL::BX + cx];
          const int x = x0 + cx, y = y0 + cy;
          if (x < nx && y < ny) {
            const int ci = (cy + TL::H) * TL::SW + TL::H + cx;
            const T u = vo[ci], lam_c = lo[ci];
            const T SP = accP[c][0] + gP[c] + sp, SMM = accM[c][0] + gM[c] + sm;
            const T au = absv(u), hu = T(0.5) * u;
            const T jt = (hu + au) * SP + (hu - au) * SMM;
            const T t = lam_c + a.dt * jt;
            const size_t o = (size_t)ko * sxy + (size_t)y * nx + x;
            if (a.stage == 3) {
              a.out[o] = T(2.0 / 3.0) * t;
              a.acc_out[o] = lam_c * T(1.0 / 3.0);
            } else if (a.stage == 2) {
              a.out[o] = T(0.25) * t;
              a.acc_out[o] = a.acc_in[o] + T(0.75) * lam_c;
            } else {
              a.out[o] = a.acc_in[o] + t;
            }
          }
        }
      }
      // shift the z accumulators: cell p-5 leaves, p+1 enters
      if (q >= 5) {
#pragma unroll
        for (int c = 0; c < 2; ++c) {
#pragma unroll
          for (int k = 0; k < 5; ++k) { accP[c][k] = accP[c][k + 1]; accM[c][k] = accM[c][k + 1]; }
          accP[c][5] = T(0);
          accM[c][5] = T(0);
        }
      }
      __syncthreads();  // slot of plane q-5 (and the face buffer) free for reuse
      if (q + TL::P + 1 < Q) issue(q + TL::P + 1);
      else cp_async_commit();
    }
  }
}

}  // namespace

// ------------------------------------------------------------------------------ host
namespace {

adv_status adjoint_validate(const adv_burgers_desc* d) {
  adv_status st = burgers_validate(d);
  if (st != ADV_OK) return st;
  if (d->bc != ADV_BC_PERIODIC || d->lf != ADV_LF_LOCAL || d->kx != 0.0 || d->ky != 0.0 || d->kz != 0.0)
    return set_error(ADV_ERR_UNSUPPORTED,
                     "burgers adjoint: periodic, local Lax-Friedrichs, inviscid schemes only");
  if (d->nz == 1) return set_error(ADV_ERR_UNSUPPORTED, "burgers adjoint: 3D grids only (nz >= 6)");
  return ADV_OK;
}

void* adjoint_kernel(const adv_burgers_desc& d) {
  const bool z = d.weno == ADV_WENO5_Z;
  if (d.dtype == ADV_F32)
    return z ? reinterpret_cast<void*>(&burgers_adjoint_kernel<float, true>)
             : reinterpret_cast<void*>(&burgers_adjoint_kernel<float, false>);
  return z ? reinterpret_cast<void*>(&burgers_adjoint_kernel<double, true>)
           : reinterpret_cast<void*>(&burgers_adjoint_kernel<double, false>);
}

template <class T>
adv_status adjoint_stage_t(const adv_burgers_desc& d, int stage, const void* v, const void* lam, const void* acc_in,
                           void* out, void* acc_out, double dt, cudaStream_t s) {
  DeviceInfo di;
  adv_status st = device_info(&di);
  if (st != ADV_OK) return st;
  AdjArgs<T> a;
  a.v = static_cast<const T*>(v);
  a.lam = static_cast<const T*>(lam);
  a.acc_in = static_cast<const T*>(acc_in);
  a.out = static_cast<T*>(out);
  a.acc_out = static_cast<T*>(acc_out);
  a.nx = d.nx; a.ny = d.ny; a.nz = d.nz;
  a.stage = stage;
  a.tiles_x = (d.nx + AdjTile::BX - 1) / AdjTile::BX;
  a.tiles_y = (d.ny + AdjTile::BY - 1) / AdjTile::BY;
  a.dt = (T)dt;
  a.rdx = (T)(1.0 / d.dx); a.rdy = (T)(1.0 / d.dy); a.rdz = (T)(1.0 / d.dz);
  void* k = adjoint_kernel(d);
  const size_t smem = AdjSmem<T>::TOTAL;
  ADV_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  ADV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 256, smem));
  occ = std::max(occ, 1);
  const int64_t units = (int64_t)a.tiles_x * a.tiles_y * d.nz;
  // four waves of equal shares, as the forward stage: later waves balance the uneven pair costs
  const int64_t ctas = std::max<int64_t>(1, std::min<int64_t>(4 * (int64_t)di.sms * occ, units / 8));
  void* args[] = {&a};
  ADV_CUDA_TRY(cudaLaunchKernel(k, dim3((unsigned)ctas), dim3(256), args, smem, s));
  count_launches(1);
  return ADV_OK;
}

adv_status adjoint_stage(const adv_burgers_desc& d, int stage, const void* v, const void* lam, const void* acc_in,
                         void* out, void* acc_out, double dt, cudaStream_t s) {
  return d.dtype == ADV_F32 ? adjoint_stage_t<float>(d, stage, v, lam, acc_in, out, acc_out, dt, s)
                            : adjoint_stage_t<double>(d, stage, v, lam, acc_in, out, acc_out, dt, s);
}

size_t one_array(const adv_burgers_desc& d) {
  return ((size_t)d.nx * d.ny * d.nz * (d.dtype == ADV_F32 ? 4 : 8) + 255) / 256 * 256;
}

// One adjoint step with scratch lamB, lamC, acc (3 arrays): lam (dJ/du^{n+1}) -> dJ/du^n.
adv_status adjoint_step(const adv_burgers_desc& d, const void* un, const void* u1, const void* u2, double dt, void* lam,
                        char* scratch, cudaStream_t s) {
  const size_t one = one_array(d);
  char* lamB = scratch;
  char* lamC = scratch + one;
  char* acc = scratch + 2 * one;
  adv_status st = adjoint_stage(d, 3, u2, lam, nullptr, lamB, acc, dt, s);
  if (st == ADV_OK) st = adjoint_stage(d, 2, u1, lamB, acc, lamC, acc, dt, s);
  if (st == ADV_OK) st = adjoint_stage(d, 1, un, lamC, acc, lam, nullptr, dt, s);
  return st;
}

// One forward step with a fixed dt from u_n into u1, u2 and u_next (u_next may be u_n).
adv_status forward_step(const adv_burgers_desc& d, const void* un, void* u1, void* u2, void* unext, double dt,
                        cudaStream_t s) {
  BurgersLaunch L;
  BurgersStageArgs a{};
  a.dt_host = dt;
  adv_status st = burgers_prepare(d, un, &L);
  a.stage = 1; a.u_in = un; a.u_n = un; a.u_out = u1;
  if (st == ADV_OK) st = burgers_launch(d, L, a, s);
  if (st == ADV_OK) st = burgers_prepare(d, u1, &L);
  a.stage = 2; a.u_in = u1; a.u_n = un; a.u_out = u2;
  if (st == ADV_OK) st = burgers_launch(d, L, a, s);
  if (st == ADV_OK) st = burgers_prepare(d, u2, &L);
  a.stage = 3; a.u_in = u2; a.u_n = un; a.u_out = unext;
  if (st == ADV_OK) st = burgers_launch(d, L, a, s);
  return st;
}

}  // namespace
}  // namespace adv

using namespace adv;

extern "C" {

adv_status adv_burgers_adjoint_step(const adv_burgers_desc* d, const void* u_n, const void* u1, const void* u2,
                                    double dt, void* lam, void* work, void* stream) {
  ADV_NVTX_RANGE("adv_burgers_adjoint_step");
  adv_status st = adjoint_validate(d);
  if (st != ADV_OK) return st;
  if (!u_n || !u1 || !u2 || !lam || !work) return set_error(ADV_ERR_INVALID_ARG, "burgers adjoint: null buffer");
  return adjoint_step(*d, u_n, u1, u2, dt, lam, static_cast<char*>(work), static_cast<cudaStream_t>(stream));
}

adv_status adv_burgers_checkpoint_bytes(const adv_burgers_desc* d, int64_t nsteps, int64_t interval,
                                        size_t* ckpt_bytes, size_t* work_bytes) {
  adv_status st = adjoint_validate(d);
  if (st != ADV_OK) return st;
  if (nsteps < 0 || interval < 1) return set_error(ADV_ERR_INVALID_ARG, "burgers adjoint: bad nsteps/interval");
  const size_t one = one_array(*d);
  const int64_t m = (nsteps + interval - 1) / interval;
  if (ckpt_bytes) *ckpt_bytes = (size_t)std::max<int64_t>(m, 1) * one;
  // backward: u1, u2 of the segment's first step, (u^n, u1, u2) of the others, 3 adjoint arrays;
  // forward: 2 stage arrays
  if (work_bytes) *work_bytes = (size_t)(3 * interval + 2) * one;
  return ADV_OK;
}

adv_status adv_burgers_forward(const adv_burgers_desc* d, void* u, double dt, int64_t nsteps, int64_t interval,
                               void* ckpt, void* work, void* stream) {
  ADV_NVTX_RANGE("adv_burgers_forward");
  adv_status st = adjoint_validate(d);
  if (st != ADV_OK) return st;
  if (!u || !work) return set_error(ADV_ERR_INVALID_ARG, "burgers adjoint: null buffer");
  if (nsteps < 0 || interval < 1 || !(dt > 0)) return set_error(ADV_ERR_INVALID_ARG, "burgers adjoint: bad nsteps/interval/dt");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t one = one_array(*d);
  const size_t nb = (size_t)d->nx * d->ny * d->nz * (d->dtype == ADV_F32 ? 4 : 8);
  char* const ub = static_cast<char*>(u);
  char* const states = static_cast<char*>(work);
  // Steps before the last checkpoint interval run in place on u through two stage arrays. The
  // last interval (with checkpoints) writes its stage inputs where adv_burgers_backward would
  // recompute them -- step r of the interval: u1 at 3r, u2 at 3r + 1, its result u^{n+1} at
  // 3r + 2 -- and its last step writes u; with interval >= nsteps the whole run is kept and the
  // backward run recomputes nothing.
  const int64_t m = (nsteps + interval - 1) / interval;
  const int64_t n_last = ckpt && nsteps > 0 ? (m - 1) * interval : nsteps;
  for (int64_t n = 0; n < nsteps; ++n) {
    if (ckpt && n % interval == 0)
      ADV_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(ckpt) + (n / interval) * one, u, nb, cudaMemcpyDeviceToDevice, s));
    if (n < n_last) {
      st = forward_step(*d, ub, states, states + one, ub, dt, s);
    } else {
      const int64_t r = n - n_last;
      const char* un = r == 0 ? ub : states + (3 * r - 1) * one;
      char* next = n + 1 < nsteps ? states + (3 * r + 2) * one : ub;
      st = forward_step(*d, un, states + 3 * r * one, states + (3 * r + 1) * one, next, dt, s);
    }
    if (st != ADV_OK) return st;
  }
  return ADV_OK;
}

adv_status adv_burgers_backward(const adv_burgers_desc* d, double dt, int64_t nsteps, int64_t interval,
                                const void* ckpt, void* lam, void* work, int flags, void* stream) {
  ADV_NVTX_RANGE("adv_burgers_backward");
  adv_status st = adjoint_validate(d);
  if (st != ADV_OK) return st;
  if (!ckpt || !lam || !work) return set_error(ADV_ERR_INVALID_ARG, "burgers adjoint: null buffer");
  if (nsteps < 0 || interval < 1 || !(dt > 0)) return set_error(ADV_ERR_INVALID_ARG, "burgers adjoint: bad nsteps/interval/dt");
  if (flags & ~ADV_BURGERS_LAST_INTERVAL_IN_WORK) return set_error(ADV_ERR_INVALID_ARG, "burgers adjoint: unknown flags");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t one = one_array(*d);
  char* states = static_cast<char*>(work);             // 3 interval - 1 arrays
  char* scratch = states + (size_t)(3 * interval - 1) * one;  // 3 arrays
  const int64_t m = (nsteps + interval - 1) / interval;
  for (int64_t seg = m - 1; seg >= 0; --seg) {
    const int64_t n0 = seg * interval, n1 = std::min(nsteps, n0 + interval);
    const char* base = static_cast<const char*>(ckpt) + seg * one;
    // step n (relative r = n - n0) keeps u^n at index 3r - 1 (the checkpoint for r = 0), u1 at
    // 3r, u2 at 3r + 1
    auto un = [&](int64_t r) -> const char* { return r == 0 ? base : states + (3 * r - 1) * one; };
    auto u1 = [&](int64_t r) { return states + (3 * r) * one; };
    auto u2 = [&](int64_t r) { return states + (3 * r + 1) * one; };
    const bool kept = seg == m - 1 && (flags & ADV_BURGERS_LAST_INTERVAL_IN_WORK);
    for (int64_t r = 0; !kept && r < n1 - n0; ++r) {
      char* next = r + 1 < n1 - n0 ? states + (3 * (r + 1) - 1) * one : nullptr;
      if (next) {
        if ((st = forward_step(*d, un(r), u1(r), u2(r), next, dt, s)) != ADV_OK) return st;
      } else {
        // the last step of the segment needs only its stage inputs: stages 1 and 2
        BurgersLaunch L;
        BurgersStageArgs a{};
        a.dt_host = dt;
        if ((st = burgers_prepare(*d, un(r), &L)) != ADV_OK) return st;
        a.stage = 1; a.u_in = un(r); a.u_n = un(r); a.u_out = u1(r);
        if ((st = burgers_launch(*d, L, a, s)) != ADV_OK) return st;
        if ((st = burgers_prepare(*d, u1(r), &L)) != ADV_OK) return st;
        a.stage = 2; a.u_in = u1(r); a.u_n = un(r); a.u_out = u2(r);
        if ((st = burgers_launch(*d, L, a, s)) != ADV_OK) return st;
      }
    }
    for (int64_t r = n1 - n0 - 1; r >= 0; --r)
      if ((st = adjoint_step(*d, un(r), u1(r), u2(r), dt, lam, scratch, s)) != ADV_OK) return st;
  }
  return ADV_OK;
}

}  // extern "C"
