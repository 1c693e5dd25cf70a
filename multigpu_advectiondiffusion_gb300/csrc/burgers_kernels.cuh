// burgers_kernels.cuh -- fused WENO5 / WENO5-Z Burgers SSP-RK3 stage for sm_103a.
//
// One launch per stage replaces the reference's five (Compute_dF, Compute_dG, Compute_dH,
// Compute_Laplace_Async, Compute_RK: SingleGPU/Burgers3d_WENO5/kernels.cu:197-530, driven by
// main.cpp:143-149) and its per-step device copy.
//
// Work layout: a CTA owns a 32 x 16 tile of x-y columns (256 threads, two rows per thread) and
// marches through a chunk of z planes. Each plane of the tile plus a 3-cell halo is staged in a
// 6-slot shared-memory ring by TMA (x start rounded down to a 16-byte boundary; periodic tiles
// at a domain edge patch their wrapped halo after the copy lands). For the output plane k:
//   * f+- of the staged plane go to shared memory once (Lax-Friedrichs split);
//   * the 33x16 x-faces and 32x17 y-faces are reconstructed by all threads in a flat loop;
//   * each thread's z-faces come from per-column register windows of f+- sliding along z;
//   * L = -(dF/dx + dG/dy + dH/dz) (+ viscous O4 term), the SSP-RK3 combine, the store and a
//     warp-shuffle max|u_out| reduction (one atomicMax per warp) for the next stage's
//     Lax-Friedrichs constant and time step all happen in the same pass.
// Every node is read from HBM once per stage and written once.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "adv_device.cuh"
#include "adv_math.cuh"
#include "weno.cuh"

namespace adv {

template <class T>
struct BurgersParams {
  const T* uin;
  const T* un;
  T* out;
  int nx, ny, nz;
  int stage;
  int periodic;  // 1: periodic wrap; 0: the reference's frozen outer 3 layers
  int bug_b2;
  int tiles_x, tiles_y;
  int tma;
  int un_is_uin;
  int lf_global;
  double dx, dy, dz;
  T kx, ky, kz;
  double dt_host, alpha_host;
  const double* dt_dev;
  const double* alpha_dev;
  const void* alpha_key;
  void* maxabs_key;
  const int* active;
  int* status;
};

struct BurgersTile {
  static constexpr int BX = 32, BY = 16, NT = 256;
  static constexpr int R = 3;
  static constexpr int PADX = 4;  // shared column 0 holds x0 - 4 (16-byte aligned for FP32 and FP64)
  static constexpr int SW = BX + 2 * PADX;  // 40
  static constexpr int SH = BY + 2 * R;     // 22
  static constexpr int PLANE = SW * SH;     // 880
  // ring: 7 slots; while plane q is consumed the slot of plane q-4 (the previous centre plane)
  // is refilled with plane q+3, so two planes stay in flight ahead of the one awaited
  static constexpr int NS = 7;
  static constexpr int P = 2;
  static constexpr int NXF = (BX + 1) * BY;  // x-faces
  static constexpr int NYF = BX * (BY + 1);  // y-faces
};

template <class T>
struct BurgersSmem {
  static constexpr int SLOT_ELEMS = ((BurgersTile::PLANE * (int)sizeof(T) + 127) / 128 * 128) / (int)sizeof(T);
  static constexpr size_t RING = (size_t)BurgersTile::NS * SLOT_ELEMS * sizeof(T);
  static constexpr size_t FPM = (size_t)BurgersTile::PLANE * sizeof(T);
  static constexpr size_t FACES = (size_t)(BurgersTile::NXF + BurgersTile::NYF) * sizeof(T);
  static constexpr size_t TOTAL = RING + 2 * FPM + FACES;
};

template <class T> __device__ __forceinline__ T absval(T v) { return fabs(v); }
template <> __device__ __forceinline__ float absval<float>(float v) { return fabsf(v); }

__device__ __forceinline__ int wrapi(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// Face reconstruction and Lax-Friedrichs split for state type T: FP32 takes the fast forms (one
// division per side, of kind D), FP64 the reference's literal operand order.
template <class T, bool Z, class D>
struct Face;
template <bool Z, class D>
struct Face<float, Z, D> {
  __device__ __forceinline__ static float f(float p0, float p1, float p2, float p3, float p4, float m0, float m1,
                                            float m2, float m3, float m4) {
    return weno_face_fast<Z, D>(p0, p1, p2, p3, p4, m0, m1, m2, m3, m4);
  }
  __device__ __forceinline__ static void split(float u, float a, float& fp, float& fm) { lf_split_fast(u, a, fp, fm); }
  // two faces / two splits at once with paired FP32 instructions (bit-identical to the above)
  __device__ __forceinline__ static float2 f2(float2 p0, float2 p1, float2 p2, float2 p3, float2 p4, float2 m0,
                                              float2 m1, float2 m2, float2 m3, float2 m4) {
    return weno_face_fast2<Z, D>(p0, p1, p2, p3, p4, m0, m1, m2, m3, m4);
  }
  __device__ __forceinline__ static void split2(float2 u, float2 a, float2& fp, float2& fm) { lf_split_fast2(u, a, fp, fm); }
};
template <bool Z, class D>
struct Face<double, Z, D> {
  __device__ __forceinline__ static double f(double p0, double p1, double p2, double p3, double p4, double m0,
                                             double m1, double m2, double m3, double m4) {
    return weno_face_ref<Z, double>(p0, p1, p2, p3, p4, m0, m1, m2, m3, m4);
  }
  __device__ __forceinline__ static void split(double u, double a, double& fp, double& fm) { lf_split<double>(u, a, fp, fm); }
};
// FP64 state with ADV_DIV_FAST: the common-denominator form, one division per side.
template <bool Z>
struct Face<double, Z, FastDiv> {
  __device__ __forceinline__ static double f(double p0, double p1, double p2, double p3, double p4, double m0,
                                             double m1, double m2, double m3, double m4) {
    return weno_face_fast64<Z>(p0, p1, p2, p3, p4, m0, m1, m2, m3, m4);
  }
  __device__ __forceinline__ static void split(double u, double a, double& fp, double& fm) { lf_split_fast64(u, a, fp, fm); }
};

struct BurgersPipe {
  int s_issue, s_wait;  // ring slots of the next plane to issue / to wait for
  unsigned parity;      // per-slot phase parity of the next wait
};

// Shared-memory objects of the Burgers pipeline (one set per CTA, whichever kernel runs it).
__device__ __forceinline__ uint64_t* burgers_bars() {
  __shared__ uint64_t bars[BurgersTile::NS];
  return bars;
}
__device__ __forceinline__ int* burgers_abort_flag() {
  __shared__ int flag;
  return &flag;
}
// A periodic edge tile's patch list: the staged plane's elements that lie outside the domain
// (slot index) and the in-plane offset of the wrapped node each takes.
struct BurgersPatch {
  int n;
  uint16_t slot[BurgersTile::PLANE];
  int64_t src[BurgersTile::PLANE];
};
static_assert(BurgersTile::PLANE <= 65535, "patch slots are 16-bit");
__device__ __forceinline__ BurgersPatch* burgers_patch() {
  __shared__ BurgersPatch patch;
  return &patch;
}

template <class T>
__device__ __forceinline__ void burgers_cta_init(const CUtensorMap* tmap, bool tma) {
  if (threadIdx.x == 0) {
    if (tma) {
      uint64_t* bars = burgers_bars();
      for (int s = 0; s < BurgersTile::NS; ++s) mbar_init(&bars[s], 1);
      mbar_fence_init();
      if (tmap) tma_prefetch_desc(tmap);
    }
    *burgers_abort_flag() = 0;
  }
  __syncthreads();
}

// One segment: output planes [zs, ze) of the column tile at (x0, y0), streamed through the
// ring. Flushes this segment's max|u_out| into p.maxabs_key. Returns the pipeline state for the
// next segment (by value, so it stays in registers), with s_issue = -1 if a wait timed out (the
// CTA must then return).
template <class T, bool Z, class D, bool VISC>
__device__ __forceinline__ BurgersPipe burgers_segment(const CUtensorMap* tmap, const BurgersParams<T>& p, int x0,
                                                       int y0, int zs, int ze, BurgersPipe pipe) {
  using TL = BurgersTile;
  using SM = BurgersSmem<T>;
  using K = typename KeyOf<T>::type;
  // FP64 (unless ADV_DIV_FAST): reference operand order, correctly rounded
  constexpr bool EXACT = sizeof(T) == 8 && !std::is_same<D, FastDiv>::value;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* ring = reinterpret_cast<T*>(smem_raw);
  T* fpS = reinterpret_cast<T*>(smem_raw + SM::RING);
  T* fmS = fpS + TL::PLANE;
  T* fxS = fmS + TL::PLANE;
  // fxS[f] for f < NXF: x-faces [BY][BX+1]; fxS[NXF + g]: y-faces [BY+1][BX]
  uint64_t* bars = burgers_bars();
  int* abort_flag = burgers_abort_flag();

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const size_t sxy = (size_t)nx * ny;
  const bool per = p.periodic != 0;

  // Lax-Friedrichs constant and dt for this stage.
  T alpha;
  if (p.alpha_dev) alpha = (T)*p.alpha_dev;
  else if (p.alpha_key) alpha = (T)key_to_value(*static_cast<const K*>(p.alpha_key));
  else alpha = (T)p.alpha_host;
  const T dt = (T)(p.dt_dev ? *p.dt_dev : p.dt_host);
  const bool glob = p.lf_global != 0;

  // This thread's share of the 1072 x/y faces of a plane: x-faces tid and tid + 256 (of 528:
  // face row f / 33, face f % 33), y-faces tid and tid + 256 (of 544: face row g / 32, column
  // g % 32), and one of the 48 left over (x-faces 512..527 in warp 0, y-faces 512..543 in warp
  // 1). base: shared-memory index of the face's first stencil value; the others follow at stride
  // 1 (x) or SW (y), known at compile time per slot, so the loads take immediate offsets.
  static_assert(TL::NXF - 2 * TL::NT == 16 && TL::NYF - 2 * TL::NT == 32, "face slots");
  auto xbase = [](int f) {
    const int row = f / (TL::BX + 1), fi = f - row * (TL::BX + 1);
    return (row + TL::R) * TL::SW + fi + 1;  // column of x0+fi-3
  };
  auto ybase = [](int g) {
    const int fj = g / TL::BX, c = g - fj * TL::BX;
    return fj * TL::SW + TL::PADX + c;  // row of y0+fj-3
  };
  const int fbx0 = xbase(tid), fbx1 = xbase(tid + TL::NT), fby0 = ybase(tid), fby1 = ybase(tid + TL::NT);
#ifdef ADV_BOUNDS_CHECK
  // every face slot's stencil (base .. base + 5 strides) inside the staged plane (CTA-uniform
  // decision, before any copy of this segment is issued)
  if (__syncthreads_or(!ADV_IN_RANGE(fbx1 + 5, TL::PLANE, p.status) ||
                       !ADV_IN_RANGE(fby1 + 5 * TL::SW, TL::PLANE, p.status)))
    return BurgersPipe{-1, -1, 0u};
#endif
  // (Reconstructing the 48 as 24 pairs in one warp, with a run-time stride, measured 2% slower:
  // one warp then carries three paired reconstructions while the others wait at the barrier.)
  const bool left_x = tid < 16, left_y = tid >= 32 && tid < 64;
  const int fbl = left_x ? xbase(2 * TL::NT + tid) : ybase(2 * TL::NT + (left_y ? tid - 32 : 0));
  // Per-thread columns: (lane, warp) and (lane, warp + 8).
  const int cx = lane;
  const int cy0 = warp, cy1 = warp + 8;
  K kmax = 0;
  const T rdx = T(1.0 / p.dx), rdy = T(1.0 / p.dy), rdz = T(1.0 / p.dz);
  const int F = per ? 0 : 3;

  int s_issue = pipe.s_issue, s_wait = pipe.s_wait;
  unsigned parity = pipe.parity;
  // z windows per column: f+ at k-2..k+2, f- at k-1..k+3, the f+ of the newest plane held back
  // one step, u at k-3..k+3 (viscous variant only).
  T fpw[2][5], fmw[2][5], fpn[2], uw[2][VISC ? 7 : 1];

  const int Q = (ze - zs) + 2 * TL::R;
  const int p0 = zs - TL::R;
  const bool edge = per && (x0 - TL::PADX < 0 || x0 + TL::BX + TL::PADX > nx || y0 - TL::R < 0 || y0 + TL::BY + TL::R > ny);
  // 2D (nz == 1): every streamed plane is the one plane, so the z faces of each column are equal
  // and their difference is exactly zero; no z layer is frozen.
  const bool twod = nz == 1;
  // Periodic plane index: within one period of the domain (the usual case) a conditional add or
  // subtract, not the integer division of wrapi (5% of the stage at 256^3).
  auto plane_z = [&](int q) {
    int z = p0 + q;
    if (per || twod) {
      if (z < 0) z += nz;
      else if (z >= nz) z -= nz;
      if ((unsigned)z >= (unsigned)nz) z = wrapi(z, nz);
    }
    return z;
  };
  // Periodic edge tile: the TMA box zero-fills what lies outside the domain. The elements to
  // patch with their wrapped neighbours are listed once per segment (CTA-uniform branch), so a
  // plane's patch is one load and one store per listed element.
  BurgersPatch* patch = burgers_patch();
  if (edge) {
    if (tid == 0) patch->n = 0;
    __syncthreads();
    for (int e = tid; e < TL::PLANE; e += TL::NT) {
      const int r = e / TL::SW, c = e - r * TL::SW;
      const int gx = x0 - TL::PADX + c, gy = y0 - TL::R + r;
      if (gx < 0 || gx >= nx || gy < 0 || gy >= ny) {
        const int k = atomicAdd(&patch->n, 1);
        patch->slot[k] = (uint16_t)e;
        patch->src[k] = (int64_t)wrapi(gy, ny) * nx + wrapi(gx, nx);
      }
    }
    __syncthreads();
  }
  auto issue = [&](int q) {
    T* dst = ring + s_issue * SM::SLOT_ELEMS;
    const int z = plane_z(q);
    if (p.tma) {
      if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        uint64_t* bar = &bars[s_issue];
        mbar_arrive_expect_tx(bar, TL::PLANE * (unsigned)sizeof(T));
        tma_load_3d(dst, tmap, x0 - TL::PADX, y0 - TL::R, z, bar);
      }
    } else {
      const bool zok = z >= 0 && z < nz;
      for (int e = tid; e < TL::PLANE; e += TL::NT) {
        const int r = e / TL::SW, c = e - r * TL::SW;
        int gx = x0 - TL::PADX + c, gy = y0 - TL::R + r;
        if (per) { gx = wrapi(gx, nx); gy = wrapi(gy, ny); }
        const bool ok = zok && gx >= 0 && gx < nx && gy >= 0 && gy < ny;
        const T* src = ok ? p.uin + (size_t)z * sxy + (size_t)gy * nx + gx : p.uin;
        cp_async_zfill<sizeof(T)>(dst + e, src, ok && ADV_IN_RANGE(src - p.uin, sxy * nz, p.status));
      }
      cp_async_commit();
    }
    s_issue = s_issue + 1 == TL::NS ? 0 : s_issue + 1;
  };

  for (int q = 0; q <= TL::P && q < Q; ++q) issue(q);
  if (!p.tma)
    for (int q = Q; q <= TL::P; ++q) cp_async_commit();

  T fz_prev[2] = {T(0), T(0)};
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    fpn[c] = T(0);
#pragma unroll
    for (int s = 0; s < 5; ++s) { fpw[c][s] = T(0); fmw[c][s] = T(0); }
#pragma unroll
    for (int s = 0; s < (VISC ? 7 : 1); ++s) uw[c][s] = T(0);
  }
  for (int q = 0; q < Q; ++q) {
    T* plq = ring + s_wait * SM::SLOT_ELEMS;
    const int s_cent = s_wait >= 3 ? s_wait - 3 : s_wait - 3 + TL::NS;  // slot of stream entry q - 3
    if (p.tma) {
      if (!mbar_wait_bounded(&bars[s_wait], (parity >> s_wait) & 1u, p.status)) *abort_flag = 1;  // every lane waits (converged)
      if (edge) {
        // the listed elements of plane q take their wrapped neighbours; written here, read only
        // after the next barrier
        const size_t zo = (size_t)plane_z(q) * sxy;
        for (int k = tid; k < patch->n; k += TL::NT) {
          const size_t gi = zo + (size_t)patch->src[k];
          const int e = patch->slot[k];
          if (ADV_IN_RANGE(gi, sxy * nz, p.status) && ADV_IN_RANGE(e, TL::PLANE, p.status)) plq[e] = p.uin[gi];
        }
      }
    } else {
      cp_async_wait<TL::P>();
    }
    // plane q visible to all threads; abort_flag uniform; and every read of stream entry q - 4
    // (the centre plane of the previous iteration) is done, so its slot can be refilled
    __syncthreads();
    const bool aborted = *abort_flag != 0;
    parity ^= 1u << s_wait;
    s_wait = s_wait + 1 == TL::NS ? 0 : s_wait + 1;
    if (p.tma) {
      if (aborted) {
        // A wait expired: let the copies already issued (planes q+1 .. q+P) land before returning.
        if (tid == 0) {
          int sl = s_wait;
          for (int m = q + 1; m < Q && m <= q + TL::P; ++m) {
            mbar_wait_bounded(&bars[sl], (parity >> sl) & 1u, p.status);
            sl = sl + 1 == TL::NS ? 0 : sl + 1;
          }
        }
        return BurgersPipe{-1, -1, 0u};
      }
      if (q + TL::P + 1 < Q) issue(q + TL::P + 1);  // into the slot of entry q - 4
    }
    // ---- z windows: push plane q for this thread's two columns
    {
      const T uq[2] = {plq[(cy0 + TL::R) * TL::SW + TL::PADX + cx], plq[(cy1 + TL::R) * TL::SW + TL::PADX + cx]};
      T fpq[2], fmq[2];
      if constexpr (sizeof(T) == 4) {
        const float2 u2 = make_float2(uq[0], uq[1]);
        const float2 a2 = glob ? f2(alpha) : make_float2(absval(uq[0]), absval(uq[1]));
        float2 fp2, fm2;
        Face<T, Z, D>::split2(u2, a2, fp2, fm2);
        fpq[0] = fp2.x; fpq[1] = fp2.y; fmq[0] = fm2.x; fmq[1] = fm2.y;
      } else {
#pragma unroll
        for (int c = 0; c < 2; ++c) Face<T, Z, D>::split(uq[c], glob ? alpha : absval(uq[c]), fpq[c], fmq[c]);
      }
#pragma unroll
      for (int c = 0; c < 2; ++c) {
#pragma unroll
        for (int s = 0; s < 4; ++s) { fpw[c][s] = fpw[c][s + 1]; fmw[c][s] = fmw[c][s + 1]; }
        fpw[c][4] = fpn[c];
        fpn[c] = fpq[c];
        fmw[c][4] = fmq[c];
        if (VISC) {
#pragma unroll
          for (int s = 0; s < 6; ++s) uw[c][s] = uw[c][s + 1];
          uw[c][VISC ? 6 : 0] = uq[c];
        }
      }
    }
    // z-face at (newest plane - 3) + 1/2 once the windows hold planes newest-5 .. newest.
    T fz_new[2] = {T(0), T(0)};
    if (q >= 5 && !twod) {  // 2D: both z faces would be equal; their difference stays exactly 0
      if constexpr (sizeof(T) == 4) {
        auto pk = [&](const T (&w)[2][5], int s) { return make_float2(w[0][s], w[1][s]); };
        const float2 fz = Face<T, Z, D>::f2(pk(fpw, 0), pk(fpw, 1), pk(fpw, 2), pk(fpw, 3), pk(fpw, 4), pk(fmw, 0),
                                            pk(fmw, 1), pk(fmw, 2), pk(fmw, 3), pk(fmw, 4));
        fz_new[0] = fz.x;
        fz_new[1] = fz.y;
      } else {
#pragma unroll
        for (int c = 0; c < 2; ++c)
          fz_new[c] = Face<T, Z, D>::f(fpw[c][0], fpw[c][1], fpw[c][2], fpw[c][3], fpw[c][4], fmw[c][0], fmw[c][1],
                                      fmw[c][2], fmw[c][3], fmw[c][4]);
      }
    }
    if (q >= 6) {
      const int k = zs + q - 6;  // output plane; its staged copy is stream entry q - 3
      const T* plc = ring + s_cent * SM::SLOT_ELEMS;
      const bool kin = per || twod || (k >= F && k < nz - F);
      const bool any_upd = kin && !aborted;
      if (any_upd) {
        // f+- of the output plane into shared memory
        if constexpr (sizeof(T) == 4) {
          // elements tid + 256 j, j = 0..3 (880 = 3 * 256 + 112), in pairs (0, 1) and (2, 3)
          static_assert(TL::PLANE > 3 * TL::NT && TL::PLANE <= 4 * TL::NT, "split pairing assumes 3..4 rounds");
#pragma unroll
          for (int j = 0; j < 4; j += 2) {
            const int e0 = tid + TL::NT * j, e1 = e0 + TL::NT;
            if (e0 >= TL::PLANE) break;
            const bool two = e1 < TL::PLANE;
            const float2 u2 = make_float2(plc[e0], two ? plc[e1] : plc[e0]);
            const float2 a2 = glob ? f2(alpha) : make_float2(absval(u2.x), absval(u2.y));
            float2 fp2, fm2;
            Face<T, Z, D>::split2(u2, a2, fp2, fm2);
            fpS[e0] = fp2.x;
            fmS[e0] = fm2.x;
            if (two) {
              fpS[e1] = fp2.y;
              fmS[e1] = fm2.y;
            }
          }
        } else {
          for (int e = tid; e < TL::PLANE; e += TL::NT) {
            const T u = plc[e];
            T fp, fm;
            Face<T, Z, D>::split(u, glob ? alpha : absval(u), fp, fm);
            fpS[e] = fp;
            fmS[e] = fm;
          }
        }
        __syncthreads();
        // x- and y-faces of the plane, this thread's precomputed share
        auto face1 = [&](int b, auto stride) {
          constexpr int st = decltype(stride)::value;
          return Face<T, Z, D>::f(fpS[b], fpS[b + st], fpS[b + 2 * st], fpS[b + 3 * st], fpS[b + 4 * st],
                                  fmS[b + st], fmS[b + 2 * st], fmS[b + 3 * st], fmS[b + 4 * st], fmS[b + 5 * st]);
        };
        using X1 = std::integral_constant<int, 1>;
        using YS = std::integral_constant<int, TL::SW>;
        if constexpr (sizeof(T) == 4) {
          // two faces per paired FP32 instruction: (x tid, x tid + 256), (y tid, y tid + 256)
          auto face2 = [&](int b0, int b1, auto stride) {
            constexpr int st = decltype(stride)::value;
            auto P = [&](int k) { return make_float2(fpS[b0 + k * st], fpS[b1 + k * st]); };
            auto M = [&](int k) { return make_float2(fmS[b0 + k * st], fmS[b1 + k * st]); };
            return Face<T, Z, D>::f2(P(0), P(1), P(2), P(3), P(4), M(1), M(2), M(3), M(4), M(5));
          };
          const float2 fx = face2(fbx0, fbx1, X1{});
          fxS[tid] = fx.x;
          fxS[tid + TL::NT] = fx.y;
          const float2 fy = face2(fby0, fby1, YS{});
          fxS[TL::NXF + tid] = fy.x;
          fxS[TL::NXF + tid + TL::NT] = fy.y;
        } else {
          fxS[tid] = face1(fbx0, X1{});
          fxS[tid + TL::NT] = face1(fbx1, X1{});
          fxS[TL::NXF + tid] = face1(fby0, YS{});
          fxS[TL::NXF + tid + TL::NT] = face1(fby1, YS{});
        }
        if (left_x) fxS[2 * TL::NT + tid] = face1(fbl, X1{});
        else if (left_y) fxS[TL::NXF + 2 * TL::NT + (tid - 32)] = face1(fbl, YS{});
        __syncthreads();
      }
      // ---- RHS, stage combine, store, max|u_out|
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int cy = c ? cy1 : cy0;
        const int x = x0 + cx, y = y0 + cy;
        const T uo = VISC ? uw[c][VISC ? 3 : 0] : plc[(cy + TL::R) * TL::SW + TL::PADX + cx];
        T res = uo;
        const bool inside = x < nx && y < ny;  // partial tiles extend past the domain
        const bool upd = any_upd && inside && (per || (x >= F && x < nx - F && y >= F && y < ny - F));
        if (upd) {
          const T fxp = fxS[cy * (TL::BX + 1) + cx + 1], fxm = fxS[cy * (TL::BX + 1) + cx];
          const T fyp = fxS[TL::NXF + (cy + 1) * TL::BX + cx], fym = fxS[TL::NXF + cy * TL::BX + cx];
          T L;
          if (EXACT) {
            L = div_rn(-sub_rn(fxp, fxm), T(p.dx));
            L = sub_rn(L, div_rn(sub_rn(fyp, fym), T(p.dy)));
            L = sub_rn(L, div_rn(sub_rn(fz_new[c], fz_prev[c]), T(p.dz)));
          } else {
            L = -(fxp - fxm) * rdx - (fyp - fym) * rdy - (fz_new[c] - fz_prev[c]) * rdz;
          }
          if (VISC) {
            const T* row = plc + (cy + TL::R) * TL::SW + TL::PADX + cx;
            constexpr int W = TL::SW;
            const T vx = sub_rn(add_rn(sub_rn(add_rn(-row[-2], mul_rn(T(16), row[-1])), mul_rn(T(30), uo)),
                                       mul_rn(T(16), row[1])), row[2]);
            const T vy = sub_rn(add_rn(sub_rn(add_rn(-row[-2 * W], mul_rn(T(16), row[-W])), mul_rn(T(30), uo)),
                                       mul_rn(T(16), row[W])), row[2 * W]);
            constexpr int Z1 = VISC ? 1 : 0, Z2 = VISC ? 2 : 0, Z4 = VISC ? 4 : 0, Z5 = VISC ? 5 : 0;
            const T vz = sub_rn(add_rn(sub_rn(add_rn(-uw[c][Z1], mul_rn(T(16), uw[c][Z2])), mul_rn(T(30), uo)),
                                       mul_rn(T(16), uw[c][Z4])), uw[c][Z5]);
            const T v = add_rn(add_rn(mul_rn(p.kx, vx), mul_rn(p.ky, vy)), mul_rn(p.kz, vz));
            L = add_rn(L, v);
            // The reference's first viscous z-block starts at slab 3 yet runs 16 slabs, adding
            // slabs 16..18 twice (kernels.cu:464-491); reproduced only on request.
            if (p.bug_b2 && !per && k >= 16 && k <= 18 && k <= nz - 3) L = add_rn(L, v);
          }
          T un;
          if (p.un_is_uin) un = uo;
          else {
            const size_t gi = (size_t)k * sxy + (size_t)y * nx + x;
            un = ADV_IN_RANGE(gi, sxy * nz, p.status) ? p.un[gi] : T(0);
          }
          res = stage_combine<T>(p.stage, un, uo, dt, L);
        }
        if (inside) {
          if (ADV_IN_RANGE((size_t)k * sxy + (size_t)y * nx + x, sxy * nz, p.status))
            p.out[(size_t)k * sxy + (size_t)y * nx + x] = res;
          const K kk = abs_key(res);
          kmax = kk > kmax ? kk : kmax;
        }
      }
    }
    if (q >= 5) {
      fz_prev[0] = fz_new[0];
      fz_prev[1] = fz_new[1];
    }
    if (!p.tma) {
      // cp.async: one commit group per plane index; the refill of entry q - 3's slot waits here
      __syncthreads();  // stream entry q - 3 fully consumed
      if (aborted) return BurgersPipe{-1, -1, 0u};
      if (q + TL::P + 1 < Q) issue(q + TL::P + 1);
      else cp_async_commit();
    }
  }
  if (p.maxabs_key) {
    kmax = warp_max(kmax);
    if (lane == 0 && kmax) atomicMax(static_cast<K*>(p.maxabs_key), kmax);
  }
  return BurgersPipe{s_issue, s_wait, parity};
}

// Minimum resident CTAs per SM the compiler must allow for (it caps registers accordingly).
// FP32 inviscid with the IEEE or FP64 weight division: asking for 2 lets the compiler pick its
// own schedule, which lands at 78-80 registers -- still three CTAs (24 warps) per SM -- and
// measured 3-4% faster than the schedule it picks under a 3-CTA bound (76 registers); the grid
// follows the occupancy it reports. FP32 with the reciprocal division and FP32 viscous: 3 (under
// a 2-CTA bound they take 86-90 registers and only two CTAs fit). FP64: 2.
template <class T, bool VISC, class D>
constexpr int burgers_min_ctas() {
  return sizeof(T) == 4 && (VISC || std::is_same<D, FastDiv>::value) ? 3 : 2;
}

template <class T, bool Z, class D, bool VISC>
__global__ void __launch_bounds__(256, burgers_min_ctas<T, VISC, D>())
burgers_stage_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ BurgersParams<T> p) {
  using TL = BurgersTile;
  if (p.active && *p.active == 0) return;
  // Balanced split: the (tile, z-plane) pairs, tile-major, are cut into gridDim.x equal
  // contiguous ranges (several waves of CTAs); a range crossing a tile boundary becomes segments.
  const int nz = p.nz;
  const int64_t total = (int64_t)p.tiles_x * p.tiles_y * nz;
  const int64_t seg_a = total * blockIdx.x / gridDim.x, seg_b = total * (blockIdx.x + 1) / gridDim.x;
  burgers_cta_init<T>(&tmap, p.tma != 0);
  BurgersPipe pipe{0, 0, 0u};
  for (int64_t pos = seg_a; pos < seg_b;) {
    const int64_t tile = pos / nz;
    const int zs = (int)(pos - tile * nz);
    const int ze = (int)min((int64_t)nz, zs + (seg_b - pos));
    pos += ze - zs;
    const int x0 = (int)(tile % p.tiles_x) * TL::BX, y0 = (int)(tile / p.tiles_x) * TL::BY;
    pipe = burgers_segment<T, Z, D, VISC>(&tmap, p, x0, y0, zs, ze, pipe);
    if (pipe.s_issue < 0) return;
  }
}

// One instance of a batched Burgers stage: the tensor map of its stage input and the stage's
// parameters (per-instance buffers, dt / Lax-Friedrichs sources, max|u| key, active flag).
template <class T>
struct alignas(64) BurgersBatchInst {
  CUtensorMap tmap;
  BurgersParams<T> p;
  int64_t unit_begin;  // first unit of this instance
  int64_t pad[7];
};

// Batched stage over many instances: the units (instance, tile, z-plane) of all instances,
// instance-major then tile-major, are cut into gridDim.x equal contiguous ranges. Instances
// whose active flag is 0 are skipped (the choice is per segment, so uniform over the CTA).
// (The batched kernel keeps three CTAs for FP32: under a 2-CTA bound it takes 120 registers.)
template <class T, bool Z, class D, bool VISC>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2)
burgers_batch_kernel(const BurgersBatchInst<T>* __restrict__ inst, int n_inst, int64_t total_units, int tma) {
  using TL = BurgersTile;
  const int64_t seg_a = total_units * blockIdx.x / gridDim.x, seg_b = total_units * (blockIdx.x + 1) / gridDim.x;
  burgers_cta_init<T>(nullptr, tma != 0);
  BurgersPipe pipe{0, 0, 0u};
  int i = 0;
  {
    int lo = 0, hi = n_inst - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (inst[mid].unit_begin <= seg_a) lo = mid; else hi = mid - 1;
    }
    i = lo;
  }
  for (int64_t pos = seg_a; pos < seg_b;) {
    while (i + 1 < n_inst && inst[i + 1].unit_begin <= pos) ++i;
    // This segment's parameters, staged in shared memory and read from there on use (as the
    // single-problem kernel reads its constant-bank parameters). A register copy spilled 168
    // bytes per thread; with this staging the ensemble ran 2.4% faster.
    __shared__ BurgersParams<T> ps;
    __syncthreads();  // every thread is done with the previous segment's parameters
    if (threadIdx.x == 0) ps = inst[i].p;
    __syncthreads();
    const BurgersParams<T>& p = ps;
    const int64_t local = pos - inst[i].unit_begin;
    const int64_t inst_end = i + 1 < n_inst ? inst[i + 1].unit_begin : total_units;
    const int64_t tile = local / p.nz;
    const int zs = (int)(local - tile * p.nz);
    const int64_t stop = min(seg_b, inst_end);
    const int ze = (int)min((int64_t)p.nz, zs + (stop - pos));
    pos += ze - zs;
    if (p.active && *p.active == 0) continue;
    const int x0 = (int)(tile % p.tiles_x) * TL::BX, y0 = (int)(tile / p.tiles_x) * TL::BY;
    const CUtensorMap* tm = &inst[i].tmap;
    if (tma && threadIdx.x == 0) tma_prefetch_desc(tm);
    pipe = burgers_segment<T, Z, D, VISC>(tm, p, x0, y0, zs, ze, pipe);
    if (pipe.s_issue < 0) return;
  }
}

}  // namespace adv
