// heat_stage.cuh -- fused heat-equation stage for sm_103a (kernel template).
//
// One launch computes a whole stage u_out = combine(u_n, u_in + dt*L(u_in)), replacing the
// reference's separate Laplacian and RK launches plus its per-step device copy
// (SingleGPU/Diffusion3d_baselineCode/kernels.cu:37-142, main.cpp:106-122;
// SingleGPU/Diffusion2d/kernels.cu:36-88).
//
// Work layout. A tile is BX x BY nodes of an x-y plane: rows of LANES threads (32, or 16 with two
// rows per warp) x one 16-byte vector each, every thread owning that vector in ROWS adjacent rows
// (2 or 4), WARPS warps per CTA. The grid is one wave of CTAs; the (tile, z-plane) pairs,
// tile-major, are split into equal contiguous ranges, one per CTA, so every SM gets the same
// work. A CTA streams its planes through a shared-memory ring: each plane of the tile plus its
// stencil halo is copied by TMA (cp.async.bulk.tensor.3d, one mbarrier per slot; the x start is
// rounded down to a 16-byte boundary, so the box is one vector wider per side). z neighbours
// come from a per-thread register window (a ring of slots addressed by constant index in an
// unrolled plane loop), y neighbours from 16-byte shared-memory rows (the thread's own rows serve
// each other), x neighbours from the thread's own vector plus warp shuffles (the first and last
// lane of a row read the halo from shared memory). Each node is read from HBM once per stage and
// written once, with 16-byte stores.
// Row pitches TMA cannot describe (not a multiple of 16 bytes, e.g. the reference's 201-node rows)
// take the same pipeline with cp.async element copies.
//
// Arithmetic. FP64 evaluates the reference's expressions operand for operand with correctly
// rounded intrinsics (no contraction). FP32 evaluates the same stencil with explicit fused
// multiply-adds in a fixed pattern (fewer instructions; the stencil is memory-bound only when the
// instruction count is low). Both are reproduced bit for bit by the CPU oracle.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "adv_device.cuh"
#include "adv_math.cuh"

namespace adv {

template <class T> struct Vec16;
template <> struct Vec16<float> { using type = float4; };
template <> struct Vec16<double> { using type = double2; };

__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float2 fma_rn(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// Tile: TX lanes per row (32, or 16 with two rows per warp) x one 16-byte vector each, RY rows per
// thread, WARPS warps.
template <class T, int ORDER, int NDIM, int ROWS = 2, int WARPS = 8, int LANES = 32>
struct HeatTile {
  static constexpr int VX = 16 / (int)sizeof(T);  // nodes per thread along x (one 16-byte vector)
  static constexpr int TX = LANES, NT = 32 * WARPS, TY = NT / TX;
  static_assert(LANES == 32 || LANES == 16, "rows of 32 or 16 lanes");
  static constexpr int RY = ROWS;  // rows per thread
  static_assert(RY * VX < 32, "node masks are 32-bit");
  static constexpr int BX = TX * VX, BY = TY * RY;
  static constexpr int R = ORDER / 2;
  static constexpr int RZ = NDIM == 3 ? R : 0;
  static constexpr int PADX = VX;  // shared column 0 holds x0 - PADX (16-byte aligned start)
  static constexpr int SW = BX + 2 * PADX;
  static constexpr int SH = BY + 2 * R;
  static constexpr int PLANE = SW * SH;
  static constexpr int PLANE_BYTES = PLANE * (int)sizeof(T);
  static constexpr int SLOT_ELEMS = ((PLANE_BYTES + 127) / 128 * 128) / (int)sizeof(T);
  static constexpr int P = NDIM == 3 ? 3 : 0;  // planes prefetched ahead of the one consumed
  static constexpr int NS = RZ + 1 + P;         // ring slots
  static constexpr size_t SMEM = (size_t)NS * SLOT_ELEMS * sizeof(T);
};

template <class T>
struct HeatParams {
  const T* uin;
  const T* un;
  T* out;
  int nx, ny, nz;
  int frozen, zero_boundary, stage;
  int tiles_x, tiles_y;
  int vec_ok;  // output rows 16-byte aligned: vector stores
  T kx, ky, kz, dt;
  int* status;  // device status word
  // Failure-path testing only (adv_test_heat_stage_withheld; read only by the kernels built with
  // HOOK = true): the TMA copy of z plane `withheld_plane` is never issued (INT_MIN: none; halo
  // planes below the grid have negative z), and the waits for planes give up after
  // `wait_limit_ns`.
  int withheld_plane;
  unsigned long long wait_limit_ns;
};

// Laplacian at one node from its neighbours along each axis (m2, m1, centre, p1, p2).
// EXACT: the reference's operand order (3D east first, kernels.cu:95-97; 2D west first,
// Diffusion2d/kernels.cu:82-83; O2 e - 2o + w, kernels.cu:58-60), correctly rounded.
// FAST (FP32): O2 fma(-2, c, p1) + m1 per axis; O4 fma(16, far-side neighbour,
// fma(-30, c, fma(16, near-side neighbour, -near-side outer))) - far-side outer with the same
// near/far sides as the reference; L = fma(kz, Sz, fma(ky, Sy, kx * Sx)).
template <class T, int ORDER, int NDIM, bool FAST>
__device__ __forceinline__ T lap(T xm2, T xm1, T c, T xp1, T xp2, T ym2, T ym1, T yp1, T yp2, T zm2, T zm1, T zp1,
                                 T zp2, T kx, T ky, T kz) {
  T Sx, Sy, Sz = bc<T>(0);
  if (ORDER == 2) {
    if (FAST) {
      Sx = add_rn(fma_rn(bc<T>(-2), c, xp1), xm1);
      Sy = add_rn(fma_rn(bc<T>(-2), c, yp1), ym1);
      if (NDIM == 3) Sz = add_rn(fma_rn(bc<T>(-2), c, zp1), zm1);
    } else {
      Sx = add_rn(sub_rn(xp1, mul_rn(bc<T>(2), c)), xm1);
      Sy = add_rn(sub_rn(yp1, mul_rn(bc<T>(2), c)), ym1);
      if (NDIM == 3) Sz = add_rn(sub_rn(zp1, mul_rn(bc<T>(2), c)), zm1);
    }
  } else {
    // near side first: +1 in 3D, -1 in 2D
    const T ax2 = NDIM == 3 ? xp2 : xm2, ax1 = NDIM == 3 ? xp1 : xm1, bx1 = NDIM == 3 ? xm1 : xp1, bx2 = NDIM == 3 ? xm2 : xp2;
    const T ay2 = NDIM == 3 ? yp2 : ym2, ay1 = NDIM == 3 ? yp1 : ym1, by1 = NDIM == 3 ? ym1 : yp1, by2 = NDIM == 3 ? ym2 : yp2;
    if (FAST) {
      Sx = sub_rn(fma_rn(bc<T>(16), bx1, fma_rn(bc<T>(-30), c, fma_rn(bc<T>(16), ax1, -ax2))), bx2);
      Sy = sub_rn(fma_rn(bc<T>(16), by1, fma_rn(bc<T>(-30), c, fma_rn(bc<T>(16), ay1, -ay2))), by2);
      if (NDIM == 3) Sz = sub_rn(fma_rn(bc<T>(16), zm1, fma_rn(bc<T>(-30), c, fma_rn(bc<T>(16), zp1, -zp2))), zm2);
    } else {
      Sx = sub_rn(add_rn(sub_rn(add_rn(-ax2, mul_rn(bc<T>(16), ax1)), mul_rn(bc<T>(30), c)), mul_rn(bc<T>(16), bx1)), bx2);
      Sy = sub_rn(add_rn(sub_rn(add_rn(-ay2, mul_rn(bc<T>(16), ay1)), mul_rn(bc<T>(30), c)), mul_rn(bc<T>(16), by1)), by2);
      if (NDIM == 3) Sz = sub_rn(add_rn(sub_rn(add_rn(-zp2, mul_rn(bc<T>(16), zp1)), mul_rn(bc<T>(30), c)), mul_rn(bc<T>(16), zm1)), zm2);
    }
  }
  if (FAST) {
    T L = fma_rn(ky, Sy, mul_rn(kx, Sx));
    if (NDIM == 3) L = fma_rn(kz, Sz, L);
    return L;
  }
  T L = add_rn(mul_rn(kx, Sx), mul_rn(ky, Sy));
  if (NDIM == 3) L = add_rn(L, mul_rn(kz, Sz));
  return L;
}

// Stage combination. EXACT: reference operand order (kernels.cu:130-138). FAST (FP32):
// 1: fma(dt, L, un); 2: fma(0.25, fma(dt, L, uin), 0.75 * un); 3: (fma(2, fma(dt, L, uin), un)) / 3.
template <class T, bool FAST>
__device__ __forceinline__ T combine(int stage, T un, T uin, T dt, T L) {
  if constexpr (!FAST) return stage_combine<T>(stage, un, uin, dt, L);
  if (stage == 2) return fma_rn(bc<T>(0.25), fma_rn(dt, L, uin), mul_rn(bc<T>(0.75), un));
  if (stage == 3) return div_rn(fma_rn(bc<T>(2), fma_rn(dt, L, uin), un), bc<T>(3));
  return fma_rn(dt, L, un);
}

// Bitwise helpers on the representation of a 4- or 8-byte value (masks are 32-bit all-ones or
// zero; an 8-byte value applies the mask to both halves).
template <class T>
__device__ __forceinline__ T bit_and(T v, unsigned m) {
  if constexpr (sizeof(T) == 4) {
    return __uint_as_float(__float_as_uint(v) & m);
  } else {
    const unsigned long long mm = ((unsigned long long)m << 32) | m;
    return __longlong_as_double((long long)((unsigned long long)__double_as_longlong(v) & mm));
  }
}
// m ? a : b per bit
template <class T>
__device__ __forceinline__ T bit_select(unsigned m, T a, T b) {
  if constexpr (sizeof(T) == 4) {
    const unsigned ua = __float_as_uint(a), ub = __float_as_uint(b);
    return __uint_as_float((ua & m) | (ub & ~m));
  } else {
    const unsigned long long mm = ((unsigned long long)m << 32) | m;
    const unsigned long long ua = (unsigned long long)__double_as_longlong(a);
    const unsigned long long ub = (unsigned long long)__double_as_longlong(b);
    return __longlong_as_double((long long)((ua & mm) | (ub & ~mm)));
  }
}

// Shared-memory pipeline of one CTA, carried across the segments it processes.
struct HeatPipe {
  int s_issue, s_wait;  // ring slots of the next plane to issue / to wait for
  unsigned parity;      // per-slot phase parity of the next wait
};

// Shared-memory objects of the heat pipeline (one set per CTA, whichever kernel runs it).
template <class T, int ORDER, int NDIM>
__device__ __forceinline__ uint64_t* heat_bars() {
  __shared__ uint64_t bars[HeatTile<T, ORDER, NDIM>::NS];
  return bars;
}
__device__ __forceinline__ int* heat_abort_flag() {
  __shared__ int flag;
  return &flag;
}

// One segment: output planes [zs, ze) of the tile at (x0, y0), streamed through the ring.
// STAGE: 1 = stage 1 / forward Euler with u_n == u_in (u_n not read); 2, 3 = RK stages;
// 0 = stage taken at run time with a separate u_n. Returns the pipeline state for the next
// segment (by value, so it stays in registers), with s_issue = -1 if a wait timed out (the CTA
// must then return).
template <class T, int ORDER, int NDIM, bool TMA, int STAGE, int ROWS = 2, int WARPS = 8, int LANES = 32,
          bool CONTRACT = false, bool HOOK = false>
__device__ __forceinline__ HeatPipe heat_segment(const CUtensorMap* tmap, const HeatParams<T>& p, int x0, int y0, int zs,
                                             int ze, HeatPipe pipe) {
  using C = HeatTile<T, ORDER, NDIM, ROWS, WARPS, LANES>;
  constexpr int RY = C::RY;
  using V = typename Vec16<T>::type;
  // FP32 always, FP64 on request: the fused multiply-add pattern instead of the reference's
  // separately rounded operations
  constexpr bool FAST = sizeof(T) == 4 || CONTRACT;
  constexpr int R = C::R, RZ = C::RZ, VX = C::VX, SW = C::SW;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* ring = reinterpret_cast<T*>(smem_raw);
  uint64_t* bars = heat_bars<T, ORDER, NDIM>();
  int* abort_flag = heat_abort_flag();
  int s_issue = pipe.s_issue, s_wait = pipe.s_wait;
  unsigned parity = pipe.parity;
  // thread coordinates in the tile from the linear thread index: a (TX, TY) block or a 1D block
  // of the same size (the mixed-width batched kernel) give the same layout
  const int tid = threadIdx.y * C::TX + threadIdx.x;
  const int tx = (int)((unsigned)tid % C::TX), ty = (int)((unsigned)tid / C::TX);
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const size_t sxy = (size_t)nx * ny;
  const int stage = STAGE == 0 ? p.stage : STAGE;
  const T kx = p.kx, ky = p.ky, kz = p.kz, dt = p.dt;
  const int F = p.frozen;
  T w[2 * RZ + 1][RY][VX];  // register window along z (w[RZ] = centre plane), re-primed per segment
  const int Q = (ze - zs) + 2 * RZ;  // planes streamed for this segment
  const int p0 = zs - RZ;            // z of stream entry 0

  auto issue = [&](int q) {
    T* dst = ring + s_issue * C::SLOT_ELEMS;
    const int z = p0 + q;
    if (TMA) {
      if (tid == 0 && (!HOOK || z != p.withheld_plane)) {
        mbar_arrive_expect_tx(&bars[s_issue], C::PLANE_BYTES);
        tma_load_3d(dst, tmap, x0 - C::PADX, y0 - R, z, &bars[s_issue]);
      }
    } else {
      const bool zok = z >= 0 && z < nz;
      for (int e = tid; e < C::PLANE; e += C::NT) {
        const int r = e / SW, c = e - r * SW;
        const int gx = x0 - C::PADX + c, gy = y0 - R + r;
        const bool ok = zok && gx >= 0 && gx < nx && gy >= 0 && gy < ny;
        const T* src = ok ? p.uin + (size_t)z * sxy + (size_t)gy * nx + gx : p.uin;
        cp_async_zfill<sizeof(T)>(dst + e, src, ok && ADV_IN_RANGE(src - p.uin, sxy * nz, p.status));
      }
      cp_async_commit();
    }
    s_issue = s_issue + 1 == C::NS ? 0 : s_issue + 1;
  };

  for (int q = 0; q <= C::P && q < Q; ++q) issue(q);
  if (!TMA)
    for (int q = Q; q <= C::P; ++q) cp_async_commit();  // one group per plane index

  const int xb = x0 + tx * VX;  // first node of this thread
  const int ya = y0 + RY * ty;  // this thread's rows: ya .. ya + RY - 1
  // Node classes of this thread's x-y positions, fixed over the segment (bit r*VX + e):
  // edge = on the outermost x/y layer (written 0 under zero_boundary), inside = in the grid.
  // Not updated on interior planes: the rows of a frozen y layer (rowkeep, bit r) and the
  // elements of a frozen x layer (xkeep, bit e; only the lanes at the x ends of the grid).
  unsigned edge = 0, inside = 0, rowkeep = 0, xkeep = 0;
#pragma unroll
  for (int r = 0; r < RY; ++r) {
    const int y = ya + r;
    if (!(y >= F && y < ny - F)) rowkeep |= 1u << r;
#pragma unroll
    for (int e = 0; e < VX; ++e) {
      const int x = xb + e;
      const unsigned bit = 1u << (r * VX + e);
      if (x == 0 || x == nx - 1 || y == 0 || y == ny - 1) edge |= bit;
      if (x < nx && y < ny) inside |= bit;
    }
  }
  // x fix-up as bit selects on the stencil result: kx_m[e] all ones on a frozen x element,
  // kx_w[e] all ones where that element keeps its input value (zero there under zero_boundary
  // on the outermost layer). Rows of a frozen y layer are fixed separately (rare warps).
  unsigned kx_m[VX], kx_w[VX];
#pragma unroll
  for (int e = 0; e < VX; ++e) {
    const int x = xb + e;
    const bool k = !(x >= F && x < nx - F);
    const bool z = p.zero_boundary && (x == 0 || x == nx - 1);
    if (k) xkeep |= 1u << e;
    kx_m[e] = k ? 0xffffffffu : 0u;
    kx_w[e] = (k && !z) ? 0xffffffffu : 0u;
  }
  constexpr unsigned ALL = (1u << (RY * VX)) - 1u;
  const bool warp_x_clean = __all_sync(0xffffffffu, xkeep == 0);
  // the common case (one frozen x layer, rows a multiple of the vector): only the first and last
  // element of a lane's vector can be frozen
  const bool warp_x_ends = __all_sync(0xffffffffu, (xkeep & ~(1u | (1u << (VX - 1)))) == 0);
  const bool warp_rows_clean = __all_sync(0xffffffffu, rowkeep == 0);
  const bool warp_inside = __all_sync(0xffffffffu, inside == ALL);
  bool row_ok[RY];
#pragma unroll
  for (int r = 0; r < RY; ++r) row_ok[r] = ya + r < ny;
  const bool vec_rows = p.vec_ok && xb + VX <= nx;
  // every lane stores whole vectors of existing rows: one uniform branch instead of one per row
  const bool warp_vec_store = __all_sync(0xffffffffu, vec_rows && ya + RY - 1 < ny);
  T* obase = p.out + (size_t)zs * sxy + (size_t)ya * nx + xb;  // output row pointer, plane zs

  // The z window is a ring of NW = 2 RZ + 1 plane slots: after ROT pushes, logical plane sl
  // (0 = oldest) sits in slot (sl + ROT) % NW. With the plane loop unrolled NW times (O2 in 3D)
  // ROT is a compile-time constant in each copy, so the window never moves between registers;
  // otherwise the slots are shifted once per plane and ROT stays 0.
  constexpr int NW = 2 * RZ + 1;
  auto plane_step = [&](auto rot, int q) -> bool {
    constexpr int ROT = decltype(rot)::value;
    auto WS = [&](int sl) -> T (&)[RY][VX] { return w[(sl + ROT) % NW]; };
    // ---- wait for plane q
    bool ok = true;
    if (TMA) {
      // every lane waits on the barrier itself (converged: same barrier, same phase)
      ok = mbar_wait_bounded(&bars[s_wait], (parity >> s_wait) & 1u, p.status, HOOK ? p.wait_limit_ns : kWaitLimitNs);
      if (!ok) *abort_flag = 1;
    } else {
      cp_async_wait<C::P>();
      __syncthreads();
    }
    parity ^= 1u << s_wait;
    const int s_cent = s_wait >= RZ ? s_wait - RZ : s_wait - RZ + C::NS;
    if (!ADV_IN_RANGE(s_wait, C::NS, p.status) || !ADV_IN_RANGE(s_cent, C::NS, p.status)) ok = false;
    const T* plq = ring + s_wait * C::SLOT_ELEMS + (RY * ty + R) * SW + C::PADX + tx * VX;
    s_wait = s_wait + 1 == C::NS ? 0 : s_wait + 1;
    const bool warp_abort = __any_sync(0xffffffffu, !ok);  // shuffles below need all lanes

    // ---- push this thread's rows of plane q into the window's newest slot
#pragma unroll
    for (int r = 0; r < RY; ++r) {
      const V v = *reinterpret_cast<const V*>(plq + r * SW);
#pragma unroll
      for (int e = 0; e < VX; ++e) WS(2 * RZ)[r][e] = reinterpret_cast<const T*>(&v)[e];
    }

    if (q >= 2 * RZ && !warp_abort) {
      const int z = p0 + q - RZ;  // output plane (stream entry q - RZ)
      const T* row0 = ring + s_cent * C::SLOT_ELEMS + (RY * ty + R) * SW + C::PADX + tx * VX;
      // x-neighbourhood of the thread's rows: xr[r][j] holds x = xb - R + j.
      T xr[RY][VX + 2 * R];
#pragma unroll
      for (int r = 0; r < RY; ++r) {
#pragma unroll
        for (int e = 0; e < VX; ++e) xr[r][R + e] = WS(RZ)[r][e];
#pragma unroll
        for (int d = 1; d <= R; ++d) {
          T lft = __shfl_up_sync(0xffffffffu, WS(RZ)[r][VX - d], 1, C::TX);
          T rgt = __shfl_down_sync(0xffffffffu, WS(RZ)[r][d - 1], 1, C::TX);
          if (tx == 0) lft = row0[r * SW - d];
          if (tx == C::TX - 1) rgt = row0[r * SW + VX - 1 + d];
          xr[r][R - d] = lft;
          xr[r][R + VX - 1 + d] = rgt;
        }
      }
      // y-neighbourhood: yv[j][e] holds row ya - R + j (j = 0 .. 2R+RY-1); rows ya .. ya+RY-1
      // are the thread's own.
      T yv[2 * R + RY][VX];
#pragma unroll
      for (int d = 1; d <= R; ++d) {
        const V a = *reinterpret_cast<const V*>(row0 - d * SW);
        const V b = *reinterpret_cast<const V*>(row0 + (RY - 1 + d) * SW);
#pragma unroll
        for (int e = 0; e < VX; ++e) {
          yv[R - d][e] = reinterpret_cast<const T*>(&a)[e];
          yv[R + RY - 1 + d][e] = reinterpret_cast<const T*>(&b)[e];
        }
      }
#pragma unroll
      for (int r = 0; r < RY; ++r)
#pragma unroll
        for (int e = 0; e < VX; ++e) yv[R + r][e] = WS(RZ)[r][e];
      const bool zin = NDIM == 2 || (z >= F && z < nz - F);
      // Every lane evaluates the stencil (halo values outside the grid are finite zero fill);
      // nodes that are not updated are fixed up afterwards with warp-uniform branches.
      T res[RY][VX];
      if constexpr (sizeof(T) == 4 && ORDER == 2) {
        // FP32 O2: node pairs (e, e+1) in paired instructions, the same operations lane by lane
        // (the O4 stencil stays scalar: paired it needs more registers than its occupancy allows)
        static_assert(VX % 2 == 0, "node pairs");
        constexpr int O1 = R >= 2 ? 2 : 1;
        const float2 kx2 = make_float2(kx, kx), ky2 = make_float2(ky, ky), kz2 = make_float2(kz, kz);
        const float2 dt2 = make_float2(dt, dt);
#pragma unroll
        for (int r = 0; r < RY; ++r)
#pragma unroll
          for (int e = 0; e < VX; e += 2) {
            auto X = [&](int j) { return make_float2(xr[r][j], xr[r][j + 1]); };
            auto Y = [&](int j) { return make_float2(yv[j][e], yv[j][e + 1]); };
            auto W = [&](int j) { return make_float2(WS(j)[r][e], WS(j)[r][e + 1]); };
            const float2 c = W(RZ);
            const float2 L = lap<float2, ORDER, NDIM, true>(
                X(R + e - O1), X(R + e - 1), c, X(R + e + 1), X(R + e + O1), Y(R + r - O1), Y(R + r - 1),
                Y(R + r + 1), Y(R + r + O1), W(RZ >= 2 ? RZ - 2 : 0), W(RZ >= 1 ? RZ - 1 : 0),
                W(RZ + (RZ >= 1 ? 1 : 0)), W(RZ + (RZ >= 2 ? 2 : 0)), kx2, ky2, kz2);
            float2 un = c;
            if (STAGE != 1) {
              const size_t off = (size_t)(q - 2 * RZ) * sxy + (size_t)r * nx + e;
              const T* src = p.un + (obase - p.out) + off;
              const bool i0 = (warp_inside || ((inside >> (r * VX + e)) & 1u)) &&
                              ADV_IN_RANGE(src - p.un, sxy * nz, p.status);
              const bool i1 = (warp_inside || ((inside >> (r * VX + e + 1)) & 1u)) &&
                              ADV_IN_RANGE(src - p.un + 1, sxy * nz, p.status);
              un = make_float2(i0 ? src[0] : T(0), i1 ? src[1] : T(0));
            }
            const float2 v = combine<float2, true>(stage, un, c, dt2, L);
            res[r][e] = v.x;
            res[r][e + 1] = v.y;
          }
      } else {
#pragma unroll
      for (int r = 0; r < RY; ++r)
#pragma unroll
        for (int e = 0; e < VX; ++e) {
          const T c = WS(RZ)[r][e];
          const T L = lap<T, ORDER, NDIM, FAST>(
              xr[r][R + e - (R >= 2 ? 2 : 1)], xr[r][R + e - 1], c, xr[r][R + e + 1], xr[r][R + e + (R >= 2 ? 2 : 1)],
              yv[R + r - (R >= 2 ? 2 : 1)][e], yv[R + r - 1][e], yv[R + r + 1][e], yv[R + r + (R >= 2 ? 2 : 1)][e],
              WS(RZ >= 2 ? RZ - 2 : 0)[r][e], WS(RZ >= 1 ? RZ - 1 : 0)[r][e], WS(RZ + (RZ >= 1 ? 1 : 0))[r][e],
              WS(RZ + (RZ >= 2 ? 2 : 0))[r][e], kx, ky, kz);
          T un = c;
          if (STAGE != 1) {
            const size_t off = (size_t)(q - 2 * RZ) * sxy + (size_t)r * nx + e;
            un = ((warp_inside || ((inside >> (r * VX + e)) & 1u)) &&
                  ADV_IN_RANGE((obase - p.out) + off, sxy * nz, p.status))
                     ? p.un[(obase - p.out) + off]
                     : T(0);
          }
          res[r][e] = combine<T, FAST>(stage, un, c, dt, L);
        }
      }
      if (!zin) {  // frozen plane: copy, or zero on the outermost planes
        const bool zero_all = p.zero_boundary && NDIM == 3 && (z == 0 || z == nz - 1);
#pragma unroll
        for (int r = 0; r < RY; ++r)
#pragma unroll
          for (int e = 0; e < VX; ++e) {
            const bool zb = zero_all || (p.zero_boundary && ((edge >> (r * VX + e)) & 1u));
            res[r][e] = zb ? T(0) : WS(RZ)[r][e];
          }
      } else {
        if (!warp_x_clean) {  // frozen x elements: res = kx_m ? (w & kx_w) : res, bitwise
          if (warp_x_ends) {
#pragma unroll
            for (int r = 0; r < RY; ++r) {
              res[r][0] = bit_select<T>(kx_m[0], bit_and<T>(WS(RZ)[r][0], kx_w[0]), res[r][0]);
              res[r][VX - 1] = bit_select<T>(kx_m[VX - 1], bit_and<T>(WS(RZ)[r][VX - 1], kx_w[VX - 1]), res[r][VX - 1]);
            }
          } else {
#pragma unroll
            for (int r = 0; r < RY; ++r)
#pragma unroll
              for (int e = 0; e < VX; ++e)
                res[r][e] = bit_select<T>(kx_m[e], bit_and<T>(WS(RZ)[r][e], kx_w[e]), res[r][e]);
          }
        }
        if (!warp_rows_clean) {  // rows of a frozen y layer: copy, or zero on the edges
#pragma unroll
          for (int r = 0; r < RY; ++r)
            if ((rowkeep >> r) & 1u)
#pragma unroll
              for (int e = 0; e < VX; ++e)
                res[r][e] = (p.zero_boundary && ((edge >> (r * VX + e)) & 1u)) ? T(0) : WS(RZ)[r][e];
        }
      }
      T* dst0 = obase + (size_t)(q - 2 * RZ) * sxy;
      if (warp_vec_store) {
#pragma unroll
        for (int r = 0; r < RY; ++r) {
          V v;
#pragma unroll
          for (int e = 0; e < VX; ++e) reinterpret_cast<T*>(&v)[e] = res[r][e];
          if (ADV_IN_RANGE(dst0 + (size_t)r * nx - p.out + VX - 1, sxy * nz, p.status))
            *reinterpret_cast<V*>(dst0 + (size_t)r * nx) = v;
        }
      } else
#pragma unroll
      for (int r = 0; r < RY; ++r) {
        if (!row_ok[r]) continue;
        T* dst = dst0 + (size_t)r * nx;
        if (vec_rows) {
          V v;
#pragma unroll
          for (int e = 0; e < VX; ++e) reinterpret_cast<T*>(&v)[e] = res[r][e];
          if (ADV_IN_RANGE(dst - p.out + VX - 1, sxy * nz, p.status)) *reinterpret_cast<V*>(dst) = v;
        } else {
#pragma unroll
          for (int e = 0; e < VX; ++e)
            if (xb + e < nx && ADV_IN_RANGE(dst + e - p.out, sxy * nz, p.status)) dst[e] = res[r][e];
        }
      }
    }
    __syncthreads();  // every read of stream entry q - RZ is done: its slot can be refilled
    if (*abort_flag) {
      // A wait expired: let every copy already issued land (bounded) before the CTA exits -- plane
      // q itself unless its copy was withheld (its slot's parity bit was already advanced), and
      // the planes prefetched after it.
      if (TMA && tid == 0) {
        const int s_q = s_wait == 0 ? C::NS - 1 : s_wait - 1;
        if (!HOOK || p0 + q != p.withheld_plane) mbar_wait_bounded(&bars[s_q], ((parity >> s_q) & 1u) ^ 1u, p.status);
        int s = s_wait;
        for (int m = q + 1; m < Q && m <= q + C::P; ++m) {
          mbar_wait_bounded(&bars[s], (parity >> s) & 1u, p.status);
          s = s + 1 == C::NS ? 0 : s + 1;
        }
      }
      return false;
    }
    if (q + C::P + 1 < Q) issue(q + C::P + 1);
    else if (!TMA) cp_async_commit();
      return true;
  };
  if constexpr (NW == 3) {
#pragma unroll 1
    for (int q = 0; q < Q; q += 3) {
      if (!plane_step(std::integral_constant<int, 0>{}, q)) return HeatPipe{-1, -1, 0u};
      if (q + 1 < Q && !plane_step(std::integral_constant<int, 1>{}, q + 1)) return HeatPipe{-1, -1, 0u};
      if (q + 2 < Q && !plane_step(std::integral_constant<int, 2>{}, q + 2)) return HeatPipe{-1, -1, 0u};
    }
  } else {
#pragma unroll 1
    for (int q = 0; q < Q; ++q) {
#pragma unroll
      for (int sl = 0; sl < NW - 1; ++sl)
#pragma unroll
        for (int r = 0; r < RY; ++r)
#pragma unroll
          for (int e = 0; e < VX; ++e) w[sl][r][e] = w[sl + 1][r][e];
      if (!plane_step(std::integral_constant<int, 0>{}, q)) return HeatPipe{-1, -1, 0u};
    }
  }
  return HeatPipe{s_issue, s_wait, parity};
}

// Resident CTAs per SM the register budget is sized for.
template <class T, int ORDER, int ROWS, int WARPS>
constexpr int heat_min_ctas() {
  return ROWS > 2 ? 16 / WARPS : (ORDER == 2 ? 4 : (sizeof(T) == 4 ? 3 : 2));
}

// HOOK: the failure-path test's variant (adv_test_heat_stage_withheld); every other launch runs the
// kernels without it.
template <class T, int ORDER, int NDIM, bool TMA, int STAGE, int ROWS = 2, int WARPS = 8, int LANES = 32,
          bool CONTRACT = false, bool HOOK = false>
__global__ void __launch_bounds__(32 * WARPS, heat_min_ctas<T, ORDER, ROWS, WARPS>())
heat_stage_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ HeatParams<T> p) {
  using C = HeatTile<T, ORDER, NDIM, ROWS, WARPS, LANES>;
  uint64_t* bars = heat_bars<T, ORDER, NDIM>();
  int& abort_flag = *heat_abort_flag();
  const int tid = threadIdx.y * C::TX + threadIdx.x;
  // Balanced split: the (tile, z-plane) pairs, tile-major, are cut into gridDim.x equal
  // contiguous ranges; a range that crosses a tile boundary becomes several segments.
  const int64_t total = (int64_t)p.tiles_x * p.tiles_y * p.nz;
  const int64_t seg_a = total * blockIdx.x / gridDim.x, seg_b = total * (blockIdx.x + 1) / gridDim.x;
  if (tid == 0) {
    if (TMA) {
      for (int s = 0; s < C::NS; ++s) mbar_init(&bars[s], 1);
      mbar_fence_init();
      tma_prefetch_desc(&tmap);
    }
    abort_flag = 0;
  }
  __syncthreads();
  HeatPipe pipe{0, 0, 0u};
  for (int64_t pos = seg_a; pos < seg_b;) {
    const int64_t tile = pos / p.nz;
    const int zs = (int)(pos - tile * p.nz);
    const int ze = (int)min((int64_t)p.nz, zs + (seg_b - pos));
    pos += ze - zs;
    const int x0 = (int)(tile % p.tiles_x) * C::BX, y0 = (int)(tile / p.tiles_x) * C::BY;
    pipe = heat_segment<T, ORDER, NDIM, TMA, STAGE, ROWS, WARPS, LANES, CONTRACT, HOOK>(&tmap, p, x0, y0, zs, ze, pipe);
    if (pipe.s_issue < 0) return;
  }
}

// One instance of a batched 3D heat run: per slot (the stages of one time step), the tensor map
// of the stage input and the stage's parameters. Forward Euler uses slots 0 (u -> w1) and
// 1 (w1 -> u); SSP-RK3 uses slots 0, 1, 2 for its three stages.
template <class T>
struct alignas(64) HeatBatchInst {
  CUtensorMap tmap[3];
  HeatParams<T> p[3];
  int64_t unit_begin;  // first unit of this instance
  int64_t pad[7];
};

// A CTA's share of a batched stage: units [u0 + units*cta/ctas, u0 + units*(cta+1)/ctas) of the
// instances inst[0 .. n_inst), whose units (instance, tile, z-plane), instance-major then
// tile-major, run from u0 (inst[0].unit_begin) to u0 + units.
template <class T, int ORDER, bool TMA, int STAGE, int ROWS, int WARPS, int LANES>
__device__ __forceinline__ void heat_batch_share(const HeatBatchInst<T>* __restrict__ inst, int n_inst, int64_t u0,
                                                 int64_t units, int cta, int ctas, int slot) {
  using C = HeatTile<T, ORDER, 3, ROWS, WARPS, LANES>;
  const int tid = threadIdx.y * C::TX + threadIdx.x;
  const int64_t seg_a = u0 + units * cta / ctas, seg_b = u0 + units * (cta + 1) / ctas;
  HeatPipe pipe{0, 0, 0u};
  // instance of the first unit (binary search on unit_begin)
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
    const HeatParams<T> p = inst[i].p[slot];  // a copy: registers, not reloads from the table
    const int64_t local = pos - inst[i].unit_begin;
    const int64_t inst_end = i + 1 < n_inst ? inst[i + 1].unit_begin : u0 + units;
    const int64_t tile = local / p.nz;
    const int zs = (int)(local - tile * p.nz);
    const int64_t stop = min(seg_b, inst_end);
    const int ze = (int)min((int64_t)p.nz, zs + (stop - pos));
    pos += ze - zs;
    const int x0 = (int)(tile % p.tiles_x) * C::BX, y0 = (int)(tile / p.tiles_x) * C::BY;
    const CUtensorMap* tm = &inst[i].tmap[slot];
    if (TMA && tid == 0) tma_prefetch_desc(tm);
    pipe = heat_segment<T, ORDER, 3, TMA, STAGE, ROWS, WARPS, LANES>(tm, p, x0, y0, zs, ze, pipe);
    if (pipe.s_issue < 0) return;
  }
}

template <class T, int ORDER, bool TMA>
__device__ __forceinline__ void heat_batch_prologue() {
  uint64_t* bars = heat_bars<T, ORDER, 3>();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    if (TMA) {
      for (int s = 0; s < HeatTile<T, ORDER, 3>::NS; ++s) mbar_init(&bars[s], 1);
      mbar_fence_init();
    }
    *heat_abort_flag() = 0;
  }
  __syncthreads();
}

// Batched stage over many 3D instances (slot `slot` of each): the units (instance, tile,
// z-plane) of all instances, instance-major then tile-major, are cut into gridDim.x equal
// contiguous ranges. Returns at once when *active == 0 (predicated steps of a device-driven
// loop).
template <class T, int ORDER, bool TMA, int STAGE, int ROWS = 2, int WARPS = 8, int LANES = 32>
__global__ void __launch_bounds__(32 * WARPS, heat_min_ctas<T, ORDER, ROWS, WARPS>())
heat_batch_kernel(const HeatBatchInst<T>* __restrict__ inst, int n_inst, int64_t total_units, int slot,
                  const int* active) {
  if (active && *active == 0) return;
  heat_batch_prologue<T, ORDER, TMA>();
  heat_batch_share<T, ORDER, TMA, STAGE, ROWS, WARPS, LANES>(inst, n_inst, 0, total_units, blockIdx.x, gridDim.x,
                                                           slot);
}

// Batched stage over instances of two tile widths (FP32 O2, TMA loads, 4 rows per thread, 4
// warps, one-dimensional blocks of 128 threads): instances [0, n_wide) in 128-wide tiles (rows
// of 32 lanes), [n_wide, n_inst) in 64-wide tiles (rows of 16 lanes), each member in the width
// that leaves fewer lanes idle on its rows. CTAs [0, ctas_wide) share the first group's units
// [0, units_wide), the others the second group's. Both tiles hold the same number of nodes and
// take the same ring (same shared memory), so a unit costs the same in either group.
template <int STAGE>
__global__ void __launch_bounds__(128, heat_min_ctas<float, 2, 4, 4>())
heat_batch_mixed_kernel(const HeatBatchInst<float>* __restrict__ inst, int n_wide, int n_inst, int64_t units_wide,
                        int64_t total_units, int ctas_wide, int slot, const int* active) {
  static_assert(HeatTile<float, 2, 3, 4, 4, 32>::SMEM == HeatTile<float, 2, 3, 4, 4, 16>::SMEM, "same ring");
  if (active && *active == 0) return;
  heat_batch_prologue<float, 2, true>();
  if ((int)blockIdx.x < ctas_wide)
    heat_batch_share<float, 2, true, STAGE, 4, 4, 32>(inst, n_wide, 0, units_wide, blockIdx.x, ctas_wide, slot);
  else
    heat_batch_share<float, 2, true, STAGE, 4, 4, 16>(inst + n_wide, n_inst - n_wide, units_wide,
                                                      total_units - units_wide, blockIdx.x - ctas_wide,
                                                      gridDim.x - ctas_wide, slot);
}

}  // namespace adv
