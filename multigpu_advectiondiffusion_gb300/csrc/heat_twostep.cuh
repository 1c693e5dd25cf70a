// heat_twostep.cuh -- two forward-Euler steps of the 3D O2 heat equation in one pass over HBM
// (FP32, sm_103a): u_out = E(E(u_in)), each E exactly the fused stage of heat_stage.cuh (same
// fused multiply-add pattern, bit for bit), replacing two launches of the reference's
// Laplacian + RK pair each (SingleGPU/Diffusion3d_baselineCode/kernels.cu:37-64, :104-142).
//
// Why: the single-step stage already runs near the HBM copy rate, so the only way to more cell
// updates per second is to move fewer bytes per update. Here each node is read once and written
// once per TWO time steps (8 B per node per launch for 2 updates instead of 16).
//
// Work layout. A CTA is 4 warps of 32 lanes; a tile is 128 x 16 nodes (one 16-byte vector of 4 nodes
// per lane, 4 rows per thread). The (tile, z-plane) pairs are cut into equal contiguous shares, one
// per CTA of a single wave, as in the single-step stage. A CTA streams the planes of its share
// along z:
//   * u planes (the input) arrive by TMA into a ring of 4 shared-memory slots, each the tile plus
//     a halo of 2 rows and one 16-byte vector per side (the halo the second step needs);
//   * at plane q the CTA computes the intermediate state v at plane q-1 on the tile plus a one-node
//     ring: its own 4 x 16 nodes per thread (z neighbours from a per-thread register window of u,
//     y from its own rows or shared memory, x from the vector and warp shuffles) and, one unit per
//     warp, the two extra rows (warps 0, 1: one vector per lane) and the two extra columns (warps
//     2, 3: one node per lane), all into a ring of 3 shared-memory v planes, and its own v into a
//     second register window;
//   * one barrier, then the final state at plane q-2 from the v window and v plane q-2, stored to
//     HBM with 16-byte stores, and the u slot of plane q-2 is refilled.
// Frozen / Dirichlet nodes keep their input (or 0 on the outermost layer) at each of the two steps,
// exactly as two single steps do. Needs rows of whole vectors (nx % 4 == 0) and the TMA path.
#pragma once
#include "heat_stage.cuh"

namespace adv {

struct Heat2Tile {
  static constexpr int VX = 4, TX = 32, WARPS = 4, NT = 32 * WARPS, TY = WARPS, RY = 4;
  static constexpr int BX = TX * VX, BY = TY * RY;   // 128 x 16 output nodes
  static constexpr int PADX = VX, SW = BX + 2 * PADX;  // shared column 0 holds x0 - 4
  static constexpr int SHU = BY + 4;                 // u rows y0-2 .. y0+BY+1
  static constexpr int SHV = BY + 2;                 // v rows y0-1 .. y0+BY
  static constexpr int U_BYTES = SW * SHU * 4;
  static constexpr int U_ELEMS = ((U_BYTES + 127) / 128 * 128) / 4;
  static constexpr int V_ELEMS = ((SW * SHV * 4 + 127) / 128 * 128) / 4;
  static constexpr int NSU = 4, NSV = 3;
  static constexpr size_t SMEM = (size_t)(NSU * U_ELEMS + NSV * V_ELEMS) * 4;
};

// Per-thread node classes of the thread's own rows (fixed over a segment), as in heat_segment:
// bit r*4+e of `edge` = the node lies on the outermost x/y layer; `rowkeep` bit r = row r lies in a
// frozen y layer; kx_m[e] all ones on a frozen x element, kx_w[e] all ones where it keeps its input
// (zero there under zero_boundary on the outermost layer).
struct Heat2Masks {
  unsigned edge, rowkeep;
  unsigned kx_m[4], kx_w[4];
  bool warp_x_clean, warp_x_ends, warp_rows_clean;
};

// The fused stencil of heat_stage.cuh (O2, 3D, FP32 fast form, stage 1 with u_n == u_in) on one
// row of 4 nodes: c = the row's vector, xl / xr = its x neighbours, ym / yp = the rows below and
// above, zm / zp = the planes below and above. Node pairs in paired instructions.
__device__ __forceinline__ void heat2_row(const float (&c)[4], float xl, float xr, const float (&ym)[4],
                                          const float (&yp)[4], const float (&zm)[4], const float (&zp)[4],
                                          float2 kx2, float2 ky2, float2 kz2, float2 dt2, float (&out)[4]) {
  const float x[6] = {xl, c[0], c[1], c[2], c[3], xr};
#pragma unroll
  for (int e = 0; e < 4; e += 2) {
    const float2 cc = make_float2(c[e], c[e + 1]);
    const float2 L = lap<float2, 2, 3, true>(cc, make_float2(x[e], x[e + 1]), cc, make_float2(x[e + 2], x[e + 3]), cc,
                                             cc, make_float2(ym[e], ym[e + 1]), make_float2(yp[e], yp[e + 1]), cc,
                                             cc, make_float2(zm[e], zm[e + 1]), make_float2(zp[e], zp[e + 1]), cc,
                                             kx2, ky2, kz2);
    const float2 v = combine<float2, true>(1, cc, cc, dt2, L);
    out[e] = v.x;
    out[e + 1] = v.y;
  }
}

// The same update on one node (the extra columns), the same operations as one lane of heat2_row.
__device__ __forceinline__ float heat2_node(float c, float xm, float xp, float ym, float yp, float zm, float zp,
                                            float kx, float ky, float kz, float dt) {
  const float L = lap<float, 2, 3, true>(c, xm, c, xp, c, c, ym, yp, c, c, zm, zp, c, kx, ky, kz);
  return combine<float, true>(1, c, c, dt, L);
}

// Frozen / Dirichlet fix-up of a thread's own rows at plane z: res = the stencil result, cen = the
// step's input at the same nodes.
__device__ __forceinline__ void heat2_fix_rows(float (&res)[4][4], const float (&cen)[4][4], const Heat2Masks& m,
                                               int z, const HeatParams<float>& p) {
  const int F = p.frozen;
  const bool zin = z >= F && z < p.nz - F;
  if (!zin) {
    const bool zero_all = p.zero_boundary && (z == 0 || z == p.nz - 1);
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const bool zb = zero_all || (p.zero_boundary && ((m.edge >> (r * 4 + e)) & 1u));
        res[r][e] = zb ? 0.f : cen[r][e];
      }
    return;
  }
  if (!m.warp_x_clean) {
    if (m.warp_x_ends) {
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        res[r][0] = bit_select<float>(m.kx_m[0], bit_and<float>(cen[r][0], m.kx_w[0]), res[r][0]);
        res[r][3] = bit_select<float>(m.kx_m[3], bit_and<float>(cen[r][3], m.kx_w[3]), res[r][3]);
      }
    } else {
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int e = 0; e < 4; ++e)
          res[r][e] = bit_select<float>(m.kx_m[e], bit_and<float>(cen[r][e], m.kx_w[e]), res[r][e]);
    }
  }
  if (!m.warp_rows_clean) {
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if ((m.rowkeep >> r) & 1u)
#pragma unroll
        for (int e = 0; e < 4; ++e)
          res[r][e] = (p.zero_boundary && ((m.edge >> (r * 4 + e)) & 1u)) ? 0.f : cen[r][e];
  }
}

// Is node (x, y, z) updated (interior), and if not, is it written as 0 (outermost layer under
// zero_boundary)? Nodes outside the grid count as frozen (their values are never read by an
// updated node).
__device__ __forceinline__ bool heat2_frozen(int x, int y, int z, const HeatParams<float>& p, bool* zero) {
  const int F = p.frozen;
  const bool in = x >= F && x < p.nx - F && y >= F && y < p.ny - F && z >= F && z < p.nz - F;
  *zero = p.zero_boundary && (x == 0 || x == p.nx - 1 || y == 0 || y == p.ny - 1 || z == 0 || z == p.nz - 1);
  return !in;
}

struct Heat2Pipe {
  int s_issue, s_wait;  // u ring slots of the next plane to issue / to wait for
  unsigned parity;      // per-slot phase parity of the next wait
};

__device__ __forceinline__ uint64_t* heat2_bars() {
  __shared__ uint64_t bars[Heat2Tile::NSU];
  return bars;
}
__device__ __forceinline__ int* heat2_abort_flag() {
  __shared__ int flag;
  return &flag;
}

// One segment: final planes [zs, ze) of the tile at (x0, y0). Returns the pipeline state for the
// next segment, with s_issue = -1 if a wait timed out (the CTA must then return).
__device__ __forceinline__ Heat2Pipe heat2_segment(const CUtensorMap* tmap, const HeatParams<float>& p, int x0, int y0,
                                                   int zs, int ze, Heat2Pipe pipe) {
  using C = Heat2Tile;
  constexpr int RY = C::RY, SW = C::SW, PADX = C::PADX;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* uring = reinterpret_cast<float*>(smem_raw);
  float* vring = uring + C::NSU * C::U_ELEMS;
  uint64_t* bars = heat2_bars();
  int* abort_flag = heat2_abort_flag();
  int s_issue = pipe.s_issue, s_wait = pipe.s_wait;
  unsigned parity = pipe.parity;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * C::TX + tx;
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const size_t sxy = (size_t)nx * ny;
  const float2 kx2 = make_float2(p.kx, p.kx), ky2 = make_float2(p.ky, p.ky), kz2 = make_float2(p.kz, p.kz);
  const float2 dt2 = make_float2(p.dt, p.dt);
  const int Q = (ze - zs) + 4;  // u planes zs-2 .. ze+1
  const int p0 = zs - 2;        // z of stream entry 0
  float wu[3][RY][4];           // u window: planes q-2, q-1, q (a ring addressed by constant index)
  float wv[3][RY][4];           // v window: planes q-3, q-2, q-1

  auto issue = [&](int q) {
    const int z = p0 + q;
    if (tid == 0 && z != p.withheld_plane) {
      mbar_arrive_expect_tx(&bars[s_issue], C::U_BYTES);
      tma_load_3d(uring + s_issue * C::U_ELEMS, tmap, x0 - PADX, y0 - 2, z, &bars[s_issue]);
    }
    s_issue = s_issue + 1 == C::NSU ? 0 : s_issue + 1;
  };
  for (int q = 0; q < C::NSU && q < Q; ++q) issue(q);

  const int xb = x0 + tx * 4;
  const int ya = y0 + RY * ty;
  Heat2Masks m;
  {
    const int F = p.frozen;
    unsigned xkeep = 0;
    m.edge = 0;
    m.rowkeep = 0;
#pragma unroll
    for (int r = 0; r < RY; ++r) {
      const int y = ya + r;
      if (!(y >= F && y < ny - F)) m.rowkeep |= 1u << r;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int x = xb + e;
        if (x == 0 || x == nx - 1 || y == 0 || y == ny - 1) m.edge |= 1u << (r * 4 + e);
      }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int x = xb + e;
      const bool k = !(x >= F && x < nx - F);
      const bool zb = p.zero_boundary && (x == 0 || x == nx - 1);
      if (k) xkeep |= 1u << e;
      m.kx_m[e] = k ? 0xffffffffu : 0u;
      m.kx_w[e] = (k && !zb) ? 0xffffffffu : 0u;
    }
    m.warp_x_clean = __all_sync(0xffffffffu, xkeep == 0);
    m.warp_x_ends = __all_sync(0xffffffffu, (xkeep & ~9u) == 0);
    m.warp_rows_clean = __all_sync(0xffffffffu, m.rowkeep == 0);
  }
  // the extra unit of this warp: warps 0 / 1 the v rows y0-1 / y0+BY (x positions as the own rows),
  // warps 2 / 3 the v columns x0-1 / x0+BX (lane l: row y0-1+l, l < BY+2)
  const int ex_row = ty == 0 ? y0 - 1 : y0 + C::BY;                 // warps 0, 1
  const int ex_col = ty == 2 ? x0 - 1 : x0 + C::BX;                 // warps 2, 3
  unsigned ex_keep = 0, ex_zero = 0;  // warps 0, 1: per element of the lane's vector
  if (ty < 2) {
    const int F = p.frozen;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int x = xb + e;
      const bool in = x >= F && x < nx - F && ex_row >= F && ex_row < ny - F;
      const bool zb = p.zero_boundary && (x == 0 || x == nx - 1 || ex_row == 0 || ex_row == ny - 1);
      if (!in) ex_keep |= 1u << e;
      if (zb) ex_zero |= 1u << e;
    }
  }
  const bool vec_store = p.vec_ok && xb + 4 <= nx;
  float* obase = p.out + (size_t)ya * nx + xb;  // output row pointer, plane 0

  auto plane_step = [&](auto rot, int q) -> bool {
    constexpr int ROT = decltype(rot)::value;
    auto WU = [&](int sl) -> float (&)[RY][4] { return wu[(sl + ROT) % 3]; };
    auto WV = [&](int sl) -> float (&)[RY][4] { return wv[(sl + ROT) % 3]; };
    // ---- wait for u plane q (every lane waits on the barrier itself)
    const bool ok = mbar_wait_bounded(&bars[s_wait], (parity >> s_wait) & 1u, p.status, p.wait_limit_ns);
    if (!ok) *abort_flag = 1;
    parity ^= 1u << s_wait;
    const int su_p = s_wait;                                   // u(q)
    const int su_c = su_p == 0 ? C::NSU - 1 : su_p - 1;       // u(q-1)
    const int su_m = su_c == 0 ? C::NSU - 1 : su_c - 1;       // u(q-2)
    s_wait = s_wait + 1 == C::NSU ? 0 : s_wait + 1;
    const bool warp_abort = __any_sync(0xffffffffu, !ok);
    const float* up = uring + su_p * C::U_ELEMS;
    const float* uc = uring + su_c * C::U_ELEMS;
    const float* um = uring + su_m * C::U_ELEMS;
    // ---- push this thread's rows of u(q) (shared rows ya-y0+2+r)
    const int urow0 = RY * ty + 2;
#pragma unroll
    for (int r = 0; r < RY; ++r) {
      const float4 v = *reinterpret_cast<const float4*>(up + (urow0 + r) * SW + PADX + tx * 4);
      WU(2)[r][0] = v.x; WU(2)[r][1] = v.y; WU(2)[r][2] = v.z; WU(2)[r][3] = v.w;
    }
    // ---- v at plane q-1 (z = p0 + q - 1)
    if (q >= 2 && !warp_abort) {
      const int zv = p0 + q - 1;
      float* vdst = vring + ((q - 1) % C::NSV) * C::V_ELEMS;
      float res[RY][4];
#pragma unroll
      for (int r = 0; r < RY; ++r) {
        float ym[4], yp[4];
        if (r == 0) {
          const float4 a = *reinterpret_cast<const float4*>(uc + (urow0 - 1) * SW + PADX + tx * 4);
          ym[0] = a.x; ym[1] = a.y; ym[2] = a.z; ym[3] = a.w;
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) ym[e] = WU(1)[r - 1][e];
        }
        if (r == RY - 1) {
          const float4 b = *reinterpret_cast<const float4*>(uc + (urow0 + RY) * SW + PADX + tx * 4);
          yp[0] = b.x; yp[1] = b.y; yp[2] = b.z; yp[3] = b.w;
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) yp[e] = WU(1)[r + 1][e];
        }
        float xl = __shfl_up_sync(0xffffffffu, WU(1)[r][3], 1);
        float xr = __shfl_down_sync(0xffffffffu, WU(1)[r][0], 1);
        if (tx == 0) xl = uc[(urow0 + r) * SW + PADX - 1];
        if (tx == 31) xr = uc[(urow0 + r) * SW + PADX + C::BX];
        heat2_row(WU(1)[r], xl, xr, ym, yp, WU(0)[r], WU(2)[r], kx2, ky2, kz2, dt2, res[r]);
      }
      heat2_fix_rows(res, WU(1), m, zv, p);
#pragma unroll
      for (int r = 0; r < RY; ++r) {
        *reinterpret_cast<float4*>(vdst + (urow0 - 1 + r) * SW + PADX + tx * 4) =
            make_float4(res[r][0], res[r][1], res[r][2], res[r][3]);
#pragma unroll
        for (int e = 0; e < 4; ++e) WV(2)[r][e] = res[r][e];
      }
      // ---- this warp's extra unit of v at plane q-1
      if (ty < 2) {
        // one extra row: shared u row ur (ur = 1 for y0-1, BY+2 for y0+BY), v row vr
        const int ur = ty == 0 ? 1 : C::BY + 2, vr = ty == 0 ? 0 : C::BY + 1;
        const int col = PADX + tx * 4;
        const float4 a = *reinterpret_cast<const float4*>(uc + ur * SW + col);
        const float4 b = *reinterpret_cast<const float4*>(uc + (ur - 1) * SW + col);
        const float4 d = *reinterpret_cast<const float4*>(uc + (ur + 1) * SW + col);
        const float4 f = *reinterpret_cast<const float4*>(um + ur * SW + col);
        const float4 g = *reinterpret_cast<const float4*>(up + ur * SW + col);
        const float c[4] = {a.x, a.y, a.z, a.w};
        const float ym[4] = {b.x, b.y, b.z, b.w}, yp[4] = {d.x, d.y, d.z, d.w};
        const float zm[4] = {f.x, f.y, f.z, f.w}, zp[4] = {g.x, g.y, g.z, g.w};
        float xl = __shfl_up_sync(0xffffffffu, c[3], 1);
        float xr = __shfl_down_sync(0xffffffffu, c[0], 1);
        if (tx == 0) xl = uc[ur * SW + PADX - 1];
        if (tx == 31) xr = uc[ur * SW + PADX + C::BX];
        float o[4];
        heat2_row(c, xl, xr, ym, yp, zm, zp, kx2, ky2, kz2, dt2, o);
        const bool zin = zv >= p.frozen && zv < nz - p.frozen;
        const bool zzero = p.zero_boundary && (zv == 0 || zv == nz - 1);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const bool keep = !zin || ((ex_keep >> e) & 1u);
          const bool zero = zzero || ((ex_zero >> e) & 1u);
          if (keep) o[e] = zero ? 0.f : c[e];
        }
        *reinterpret_cast<float4*>(vdst + vr * SW + col) = make_float4(o[0], o[1], o[2], o[3]);
      } else if (tx < C::SHV) {
        // one extra column: lane l is v row l (y = y0-1+l), shared u row l+1, column uc_col
        const int col = ty == 2 ? PADX - 1 : PADX + C::BX;
        const int ur = tx + 1;
        const float c = uc[ur * SW + col];
        float o = heat2_node(c, uc[ur * SW + col - 1], uc[ur * SW + col + 1], uc[(ur - 1) * SW + col],
                             uc[(ur + 1) * SW + col], um[ur * SW + col], up[ur * SW + col], p.kx, p.ky, p.kz, p.dt);
        bool zero;
        if (heat2_frozen(ex_col, y0 - 1 + tx, zv, p, &zero)) o = zero ? 0.f : c;
        vdst[tx * SW + col] = o;
      }
    }
    __syncthreads();  // v(q-1) visible; every read of u(q-2) done: its slot can be refilled
    if (*abort_flag) {
      // A wait expired: let every copy already issued land (bounded) before the CTA exits -- plane
      // q itself unless its copy was withheld, and the planes issued after it (up to q + 1, or the
      // initial fill of the ring). Slot su_p's parity bit was already advanced past plane q.
      if (tid == 0) {
        const int last = min(Q - 1, max(C::NSU - 1, q + 1));
        const unsigned par = parity ^ (1u << su_p);
        int s = su_p;
        for (int n = q; n <= last; ++n) {
          if (p0 + n != p.withheld_plane) mbar_wait_bounded(&bars[s], (par >> s) & 1u, p.status);
          s = s + 1 == C::NSU ? 0 : s + 1;
        }
      }
      return false;
    }
    if (q >= 2 && q + 2 < Q) issue(q + 2);
    // ---- final state at plane q-2 (z = p0 + q - 2) from v(q-3), v(q-2), v(q-1)
    if (q >= 4) {
      const int zw = p0 + q - 2;
      const float* vc = vring + ((q - 2) % C::NSV) * C::V_ELEMS;
      const int vrow0 = RY * ty + 1;  // shared v row of this thread's first row
      float res[RY][4];
#pragma unroll
      for (int r = 0; r < RY; ++r) {
        float ym[4], yp[4];
        if (r == 0) {
          const float4 a = *reinterpret_cast<const float4*>(vc + (vrow0 - 1) * SW + PADX + tx * 4);
          ym[0] = a.x; ym[1] = a.y; ym[2] = a.z; ym[3] = a.w;
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) ym[e] = WV(1)[r - 1][e];
        }
        if (r == RY - 1) {
          const float4 b = *reinterpret_cast<const float4*>(vc + (vrow0 + RY) * SW + PADX + tx * 4);
          yp[0] = b.x; yp[1] = b.y; yp[2] = b.z; yp[3] = b.w;
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) yp[e] = WV(1)[r + 1][e];
        }
        float xl = __shfl_up_sync(0xffffffffu, WV(1)[r][3], 1);
        float xr = __shfl_down_sync(0xffffffffu, WV(1)[r][0], 1);
        if (tx == 0) xl = vc[(vrow0 + r) * SW + PADX - 1];
        if (tx == 31) xr = vc[(vrow0 + r) * SW + PADX + C::BX];
        heat2_row(WV(1)[r], xl, xr, ym, yp, WV(0)[r], WV(2)[r], kx2, ky2, kz2, dt2, res[r]);
      }
      heat2_fix_rows(res, WV(1), m, zw, p);
      float* dst0 = obase + (size_t)zw * sxy;
      if (vec_store) {
#pragma unroll
        for (int r = 0; r < RY; ++r)
          if (ya + r < ny)
            *reinterpret_cast<float4*>(dst0 + (size_t)r * nx) = make_float4(res[r][0], res[r][1], res[r][2], res[r][3]);
      }
    }
    return true;
  };
#pragma unroll 1
  for (int q = 0; q < Q; q += 3) {
    if (!plane_step(std::integral_constant<int, 0>{}, q)) return Heat2Pipe{-1, -1, 0u};
    if (q + 1 < Q && !plane_step(std::integral_constant<int, 1>{}, q + 1)) return Heat2Pipe{-1, -1, 0u};
    if (q + 2 < Q && !plane_step(std::integral_constant<int, 2>{}, q + 2)) return Heat2Pipe{-1, -1, 0u};
  }
  return Heat2Pipe{s_issue, s_wait, parity};
}

__global__ void __launch_bounds__(Heat2Tile::NT, 3)
heat_twostep_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ HeatParams<float> p) {
  using C = Heat2Tile;
  uint64_t* bars = heat2_bars();
  int& abort_flag = *heat2_abort_flag();
  const int tid = threadIdx.y * C::TX + threadIdx.x;
  const int64_t total = (int64_t)p.tiles_x * p.tiles_y * p.nz;
  const int64_t seg_a = total * blockIdx.x / gridDim.x, seg_b = total * (blockIdx.x + 1) / gridDim.x;
  if (tid == 0) {
    for (int s = 0; s < C::NSU; ++s) mbar_init(&bars[s], 1);
    mbar_fence_init();
    tma_prefetch_desc(&tmap);
    abort_flag = 0;
  }
  __syncthreads();
  Heat2Pipe pipe{0, 0, 0u};
  for (int64_t pos = seg_a; pos < seg_b;) {
    const int64_t tile = pos / p.nz;
    const int zs = (int)(pos - tile * p.nz);
    const int ze = (int)min((int64_t)p.nz, zs + (seg_b - pos));
    pos += ze - zs;
    const int x0 = (int)(tile % p.tiles_x) * C::BX, y0 = (int)(tile / p.tiles_x) * C::BY;
    pipe = heat2_segment(&tmap, p, x0, y0, zs, ze, pipe);
    if (pipe.s_issue < 0) return;
  }
}

}  // namespace adv
