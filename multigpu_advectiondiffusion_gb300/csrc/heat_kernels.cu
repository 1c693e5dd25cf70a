// heat_kernels.cu -- fused heat-equation stage for sm_103a.
//
// One launch computes a whole stage u_out = combine(u_n, u_in + dt*L(u_in)), replacing the
// reference's separate Laplacian and RK launches plus its per-step device copy
// (SingleGPU/Diffusion3d_baselineCode/kernels.cu:37-142, main.cpp:106-122;
// SingleGPU/Diffusion2d/kernels.cu:36-88).
//
// Layout of the work: a CTA owns an x-y tile of BX x BY nodes (BX = 32 lanes x one 16-byte
// vector per lane) and marches through a chunk of z planes. Each plane of the tile plus its
// stencil halo is staged into a shared-memory ring by TMA (cp.async.bulk.tensor.3d with an
// mbarrier per slot; the x start is rounded down to a 16-byte boundary, so the box is widened
// by one vector on each side). x/y neighbours come from the staged plane, z neighbours from a
// per-thread register window that slides along z, so each node is read from HBM once per stage.
// Strides that TMA cannot describe (row pitch not a multiple of 16 bytes, e.g. the reference's
// 201 x 199 x 200 grid) take the same pipeline with cp.async element copies instead.
// Arithmetic uses correctly rounded intrinsics in the reference's operand order, so FP32/FP64
// results equal the CPU oracle's bit for bit.
#include <algorithm>
#include <cstring>

#include "adv_device.cuh"
#include "adv_internal.h"
#include "adv_math.cuh"

namespace adv {

template <class T> struct Vec16;
template <> struct Vec16<float> { using type = float4; };
template <> struct Vec16<double> { using type = double2; };

template <class T, int ORDER, int NDIM>
struct HeatTile {
  static constexpr int VX = 16 / (int)sizeof(T);  // nodes per thread along x (one 16-byte vector)
  static constexpr int TX = 32, TY = 8, NT = TX * TY;
  static constexpr int BX = TX * VX, BY = TY;
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
  int zchunk;
  int un_is_uin;  // stage input equals u_n: the centre value is reused, u_n is not read
  int vec_ok;     // rows are 16-byte aligned: vector stores
  T kx, ky, kz, dt;
  int* status;  // device status word
};

template <class T, int ORDER, int NDIM, bool TMA>
__global__ void __launch_bounds__(256)
heat_stage_kernel(const __grid_constant__ CUtensorMap tmap, const HeatParams<T> p) {
  using C = HeatTile<T, ORDER, NDIM>;
  using V = typename Vec16<T>::type;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* ring = reinterpret_cast<T*>(smem_raw);
  __shared__ uint64_t bars[C::NS];
  __shared__ int abort_flag;

  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * C::TX + tx;
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const int x0 = blockIdx.x * C::BX, y0 = blockIdx.y * C::BY;
  const int zs = NDIM == 3 ? (int)blockIdx.z * p.zchunk : 0;
  const int ze = NDIM == 3 ? min(nz, zs + p.zchunk) : 1;
  const int Q = (ze - zs) + 2 * C::RZ;  // planes streamed by this CTA
  const int p0 = zs - C::RZ;            // z of stream entry 0
  const size_t sxy = (size_t)nx * ny;

  if (tid == 0) {
    if (TMA) {
      for (int s = 0; s < C::NS; ++s) mbar_init(&bars[s], 1);
      mbar_fence_init();
      tma_prefetch_desc(&tmap);
    }
    abort_flag = 0;
  }
  __syncthreads();

  auto issue = [&](int q) {
    T* dst = ring + (q % C::NS) * C::SLOT_ELEMS;
    const int z = p0 + q;
    if (TMA) {
      if (tid == 0) {
        uint64_t* bar = &bars[q % C::NS];
        mbar_arrive_expect_tx(bar, C::PLANE_BYTES);
        tma_load_3d(dst, &tmap, x0 - C::PADX, y0 - C::R, z, bar);
      }
    } else {
      const bool zok = z >= 0 && z < nz;
      for (int e = tid; e < C::PLANE; e += C::NT) {
        const int r = e / C::SW, c = e - r * C::SW;
        const int gx = x0 - C::PADX + c, gy = y0 - C::R + r;
        const bool ok = zok && gx >= 0 && gx < nx && gy >= 0 && gy < ny;
        const T* src = ok ? p.uin + (size_t)z * sxy + (size_t)gy * nx + gx : p.uin;
        cp_async_zfill<sizeof(T)>(dst + e, src, ok);
      }
    }
  };

  // prologue: planes 0..P
  for (int q = 0; q <= C::P && q < Q; ++q) {
    issue(q);
    if (!TMA) cp_async_commit();
  }
  if (!TMA)
    for (int q = Q; q <= C::P; ++q) cp_async_commit();  // keep one group per plane index

  const T kx = p.kx, ky = p.ky, kz = p.kz, dt = p.dt;
  const int F = p.frozen;
  const int xb = x0 + tx * C::VX;  // first node of this thread
  const int y = y0 + ty;
  T w[2 * C::RZ + 1][C::VX];       // register window along z: w[RZ] is the centre plane

  for (int q = 0; q < Q; ++q) {
    // ---- wait for plane q
    if (TMA) {
      if (!mbar_wait_bounded(&bars[q % C::NS], (q / C::NS) & 1, p.status)) abort_flag = 1;
    } else {
      cp_async_wait<C::P>();
      __syncthreads();
    }
    const T* plq = ring + (q % C::NS) * C::SLOT_ELEMS;
    // ---- slide the window and push this thread's nodes of plane q
#pragma unroll
    for (int s = 0; s < 2 * C::RZ; ++s)
#pragma unroll
      for (int e = 0; e < C::VX; ++e) w[s][e] = w[s + 1][e];
    {
      const V v = *reinterpret_cast<const V*>(plq + (ty + C::R) * C::SW + C::PADX + tx * C::VX);
      const T* vv = reinterpret_cast<const T*>(&v);
#pragma unroll
      for (int e = 0; e < C::VX; ++e) w[2 * C::RZ][e] = vv[e];
    }

    if (q >= 2 * C::RZ && !abort_flag) {
      // ---- output plane z = p0 + q - RZ, staged at stream entry q - RZ
      const int z = p0 + q - C::RZ;
      const T* pc = ring + ((q - C::RZ) % C::NS) * C::SLOT_ELEMS;
      const T* row = pc + (ty + C::R) * C::SW + C::PADX + tx * C::VX;
      T res[C::VX];
      const bool zin = NDIM == 2 || (z >= F && z < nz - F);
      const bool zouter = NDIM == 3 && (z == 0 || z == nz - 1);
      const bool yin = y >= F && y < ny - F;
      const bool youter = y == 0 || y == ny - 1;
#pragma unroll
      for (int e = 0; e < C::VX; ++e) {
        const int x = xb + e;
        const T uo = w[C::RZ][e];
        const bool upd = zin && yin && x >= F && x < nx - F;
        if (upd) {
          T L;
          if (ORDER == 4) {
            // Operand order of the reference: east/north first in 3D (Diffusion3d_baselineCode/
            // kernels.cu:95-97), west/south first in 2D (Diffusion2d/kernels.cu:82-83).
            constexpr int D1 = NDIM == 3 ? 1 : -1, D2 = 2 * D1;
            const T Sx = sub_rn(add_rn(sub_rn(add_rn(-row[e + D2], mul_rn(T(16), row[e + D1])), mul_rn(T(30), uo)),
                                       mul_rn(T(16), row[e - D1])), row[e - D2]);
            const T Sy = sub_rn(add_rn(sub_rn(add_rn(-row[e + D2 * C::SW], mul_rn(T(16), row[e + D1 * C::SW])), mul_rn(T(30), uo)),
                                       mul_rn(T(16), row[e - D1 * C::SW])), row[e - D2 * C::SW]);
            L = add_rn(mul_rn(kx, Sx), mul_rn(ky, Sy));
            if (NDIM == 3) {
              constexpr int ZP2 = NDIM == 3 ? 2 * C::RZ : 0, ZP1 = NDIM == 3 ? C::RZ + 1 : 0;
              constexpr int ZM1 = NDIM == 3 ? C::RZ - 1 : 0;
              const T Sz = sub_rn(add_rn(sub_rn(add_rn(-w[ZP2][e], mul_rn(T(16), w[ZP1][e])), mul_rn(T(30), uo)),
                                         mul_rn(T(16), w[ZM1][e])),
                                  w[0][e]);
              L = add_rn(L, mul_rn(kz, Sz));
            }
          } else {
            const T Sx = add_rn(sub_rn(row[e + 1], mul_rn(T(2), uo)), row[e - 1]);
            const T Sy = add_rn(sub_rn(row[e + C::SW], mul_rn(T(2), uo)), row[e - C::SW]);
            L = add_rn(mul_rn(kx, Sx), mul_rn(ky, Sy));
            if (NDIM == 3) {
              const T Sz = add_rn(sub_rn(w[2 * C::RZ][e], mul_rn(T(2), uo)), w[0][e]);
              L = add_rn(L, mul_rn(kz, Sz));
            }
          }
          T un;
          if (p.un_is_uin) un = uo;
          else {
            const bool inb = x < nx && y < ny;
            un = inb ? p.un[(size_t)z * sxy + (size_t)y * nx + x] : T(0);
          }
          res[e] = stage_combine<T>(p.stage, un, uo, dt, L);
        } else {
          const bool outer = youter || zouter || x == 0 || x == nx - 1;
          res[e] = (p.zero_boundary && outer) ? T(0) : uo;
        }
      }
      if (y < ny) {
        T* dst = p.out + (size_t)z * sxy + (size_t)y * nx + xb;
        if (p.vec_ok && xb + C::VX <= nx) {
          V v;
          T* vv = reinterpret_cast<T*>(&v);
#pragma unroll
          for (int e = 0; e < C::VX; ++e) vv[e] = res[e];
          *reinterpret_cast<V*>(dst) = v;
        } else {
#pragma unroll
          for (int e = 0; e < C::VX; ++e)
            if (xb + e < nx) dst[e] = res[e];
        }
      }
    }
    __syncthreads();  // every read of stream entry q - RZ is done: its slot can be refilled
    if (abort_flag) {
      // A wait expired: let the copies already issued land (bounded) before the CTA exits.
      if (TMA && tid == 0)
        for (int m = q; m < Q && m <= q + C::P; ++m) mbar_wait_bounded(&bars[m % C::NS], (m / C::NS) & 1, p.status);
      return;
    }
    if (q + C::P + 1 < Q) issue(q + C::P + 1);
    if (!TMA) cp_async_commit();
  }
}

// ----------------------------------------------------------------------------- host side

adv_status heat_validate(const adv_heat_desc* d) {
  if (!d) return set_error(ADV_ERR_INVALID_ARG, "heat: null descriptor");
  if (d->ndim != 2 && d->ndim != 3) return set_error(ADV_ERR_INVALID_ARG, "heat: ndim must be 2 or 3");
  if (d->dtype != ADV_F32 && d->dtype != ADV_F64) return set_error(ADV_ERR_INVALID_ARG, "heat: bad dtype");
  if (d->order != 2 && d->order != 4) return set_error(ADV_ERR_INVALID_ARG, "heat: order must be 2 or 4");
  const int nzv = d->ndim == 3 ? d->nz : 1;
  if (d->nx < 1 || d->ny < 1 || nzv < 1) return set_error(ADV_ERR_INVALID_ARG, "heat: empty grid");
  if (d->ndim == 2 && d->nz != 1) return set_error(ADV_ERR_INVALID_ARG, "heat: nz must be 1 in 2D");
  if (d->frozen < d->order / 2)
    return set_error(ADV_ERR_INVALID_ARG, "heat: frozen layers must cover the stencil radius");
  if ((int64_t)d->nx * d->ny * nzv > (int64_t)1 << 40) return set_error(ADV_ERR_INVALID_ARG, "heat: grid too large");
  if (d->nx > (1 << 30) || d->ny > (1 << 30) || nzv > (1 << 30))
    return set_error(ADV_ERR_INVALID_ARG, "heat: dimension too large");
  return ADV_OK;
}

namespace {

template <class T, int ORDER, int NDIM, bool TMA>
void* heat_kernel_ptr() {
  return reinterpret_cast<void*>(&heat_stage_kernel<T, ORDER, NDIM, TMA>);
}

void* pick_kernel(int dtype, int order, int ndim, bool tma) {
#define PICK(T, O, N)                                                                   \
  if (order == O && ndim == N)                                                          \
    return tma ? heat_kernel_ptr<T, O, N, true>() : heat_kernel_ptr<T, O, N, false>();
  if (dtype == ADV_F32) {
    PICK(float, 2, 3) PICK(float, 4, 3) PICK(float, 2, 2) PICK(float, 4, 2)
  } else {
    PICK(double, 2, 3) PICK(double, 4, 3) PICK(double, 2, 2) PICK(double, 4, 2)
  }
#undef PICK
  return nullptr;
}

template <class T, int ORDER, int NDIM>
void tile_dims(int* bx, int* by, int* sw, int* sh, int* padx, int* r, size_t* smem) {
  using C = HeatTile<T, ORDER, NDIM>;
  *bx = C::BX; *by = C::BY; *sw = C::SW; *sh = C::SH; *padx = C::PADX; *r = C::R; *smem = C::SMEM;
}

void tile_for(int dtype, int order, int ndim, int* bx, int* by, int* sw, int* sh, int* padx, int* r,
              size_t* smem) {
#define TD(T, O, N) if (order == O && ndim == N) return tile_dims<T, O, N>(bx, by, sw, sh, padx, r, smem);
  if (dtype == ADV_F32) { TD(float, 2, 3) TD(float, 4, 3) TD(float, 2, 2) TD(float, 4, 2) }
  else { TD(double, 2, 3) TD(double, 4, 3) TD(double, 2, 2) TD(double, 4, 2) }
#undef TD
}

}  // namespace

adv_status heat_prepare(const adv_heat_desc& d, const void* u_in, HeatLaunch* L) {
  DeviceInfo di;
  adv_status st = device_info(&di);
  if (st != ADV_OK) return st;
  int bx, by, sw, sh, padx, r;
  size_t smem;
  tile_for(d.dtype, d.order, d.ndim, &bx, &by, &sw, &sh, &padx, &r, &smem);
  const int es = d.dtype == ADV_F32 ? 4 : 8;
  const int nz = d.ndim == 3 ? d.nz : 1;
  // TMA needs 16-byte aligned base and strides.
  const bool aligned = ((uintptr_t)u_in % 16 == 0) && (((int64_t)d.nx * es) % 16 == 0) &&
                       (((int64_t)d.nx * d.ny * es) % 16 == 0);
  L->tma = aligned;
  L->block = dim3(32, 8, 1);
  const int tiles_x = (d.nx + bx - 1) / bx, tiles_y = (d.ny + by - 1) / by;
  int zchunk = 1;
  if (d.ndim == 3) {
    // Enough CTAs for ~4 per SM, but z-chunks of at least 8 planes so the z halo stays small.
    const int64_t want = (int64_t)di.sms * 4;
    int64_t chunks = (want + (int64_t)tiles_x * tiles_y - 1) / ((int64_t)tiles_x * tiles_y);
    chunks = std::max<int64_t>(1, std::min<int64_t>(chunks, (nz + 7) / 8));
    zchunk = (int)((nz + chunks - 1) / chunks);
  }
  L->zchunk = zchunk;
  L->grid = dim3(tiles_x, tiles_y, d.ndim == 3 ? (nz + zchunk - 1) / zchunk : 1);
  L->smem = smem;
  void* k = pick_kernel(d.dtype, d.order, d.ndim, L->tma);
  if (!k) return set_error(ADV_ERR_UNSUPPORTED, "heat: no kernel for this configuration");
  ADV_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  std::memset(&L->tmap_in, 0, sizeof(L->tmap_in));
  if (L->tma) {
    EncodeTiledFn enc = encode_tiled_fn();
    if (!enc) return set_error(ADV_ERR_CUDA, "heat: cuTensorMapEncodeTiled unavailable");
    cuuint64_t gdim[3] = {(cuuint64_t)d.nx, (cuuint64_t)d.ny, (cuuint64_t)nz};
    cuuint64_t gstride[2] = {(cuuint64_t)d.nx * es, (cuuint64_t)d.nx * d.ny * es};
    cuuint32_t box[3] = {(cuuint32_t)sw, (cuuint32_t)sh, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult cr = enc(&L->tmap_in, d.dtype == ADV_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                      3, const_cast<void*>(u_in), gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return set_error(ADV_ERR_CUDA, "heat: cuTensorMapEncodeTiled failed");
  }
  return ADV_OK;
}

template <class T>
static adv_status heat_launch_t(const adv_heat_desc& d, const HeatLaunch& L, int stage, const void* u_in,
                                const void* u_n, void* u_out, cudaStream_t s) {
  HeatParams<T> p;
  p.uin = static_cast<const T*>(u_in);
  p.un = static_cast<const T*>(u_n);
  p.out = static_cast<T*>(u_out);
  p.nx = d.nx; p.ny = d.ny; p.nz = d.ndim == 3 ? d.nz : 1;
  p.frozen = d.frozen; p.zero_boundary = d.zero_boundary; p.stage = stage;
  p.zchunk = L.zchunk;
  p.un_is_uin = (u_n == u_in) ? 1 : 0;
  p.vec_ok = (((uintptr_t)u_out % 16) == 0 && ((int64_t)d.nx * sizeof(T)) % 16 == 0) ? 1 : 0;
  p.kx = (T)d.kx; p.ky = (T)d.ky; p.kz = (T)d.kz; p.dt = (T)d.dt;
  p.status = device_status_ptr();
  void* k = pick_kernel(d.dtype, d.order, d.ndim, L.tma);
  void* args[] = {const_cast<CUtensorMap*>(&L.tmap_in), &p};
  ADV_CUDA_TRY(cudaLaunchKernel(k, L.grid, L.block, args, L.smem, s));
  count_launches(1);
  return ADV_OK;
}

adv_status heat_launch(const adv_heat_desc& d, const HeatLaunch& L, int stage, const void* u_in, const void* u_n,
                       void* u_out, cudaStream_t s) {
  if (stage < 1 || stage > 3) return set_error(ADV_ERR_INVALID_ARG, "heat: stage must be 1, 2 or 3");
  if (d.dtype == ADV_F32) return heat_launch_t<float>(d, L, stage, u_in, u_n, u_out, s);
  return heat_launch_t<double>(d, L, stage, u_in, u_n, u_out, s);
}

}  // namespace adv
