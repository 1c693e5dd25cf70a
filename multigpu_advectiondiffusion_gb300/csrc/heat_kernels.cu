// heat_kernels.cu -- host side of the fused heat stage: validation, launch sizing, tensor maps.
// The kernel itself is heat_stage.cuh, instantiated per precision in heat_f32.cu / heat_f64.cu.
#include <algorithm>
#include <cstring>

#include "heat_launch.cuh"

namespace adv {

void* heat_kernel_f32(int order, int ndim, bool tma, int stage_kind, int rows, int warps, int lanes);
void* heat_kernel_f64(int order, int ndim, bool tma, int stage_kind, int rows, int warps, int lanes, bool contract);

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
  if (d->contract != 0 && d->contract != 1) return set_error(ADV_ERR_INVALID_ARG, "heat: contract must be 0 or 1");
  if (d->nx > (1 << 30) || d->ny > (1 << 30) || nzv > (1 << 30))
    return set_error(ADV_ERR_INVALID_ARG, "heat: dimension too large");
  return ADV_OK;
}

namespace {

void* pick_kernel(const adv_heat_desc& d, bool tma, int stage_kind, const HeatLaunch& L) {
  return d.dtype == ADV_F32 ? heat_kernel_f32(d.order, d.ndim, tma, stage_kind, L.rows, L.warps, L.lanes)
                            : heat_kernel_f64(d.order, d.ndim, tma, stage_kind, L.rows, L.warps, L.lanes,
                                              d.contract != 0);
}

template <class T, int ORDER, int NDIM, int ROWS, int WARPS = 8, int LANES = 32>
void tile_dims(int* bx, int* by, int* sw, int* sh, int* padx, int* r, size_t* smem) {
  using C = HeatTile<T, ORDER, NDIM, ROWS, WARPS, LANES>;
  *bx = C::BX; *by = C::BY; *sw = C::SW; *sh = C::SH; *padx = C::PADX; *r = C::R; *smem = C::SMEM;
}

void tile_for(int dtype, int order, int ndim, int rows, int lanes, int* bx, int* by, int* sw, int* sh, int* padx,
              int* r, size_t* smem) {
  if (rows == 4 && lanes == 16) return tile_dims<float, 2, 3, 4, 4, 16>(bx, by, sw, sh, padx, r, smem);
  if (rows == 4) return tile_dims<float, 2, 3, 4, 4, 32>(bx, by, sw, sh, padx, r, smem);
#define TD(T, O, N) if (order == O && ndim == N) return tile_dims<T, O, N, 2>(bx, by, sw, sh, padx, r, smem);
  if (dtype == ADV_F32) { TD(float, 2, 3) TD(float, 4, 3) TD(float, 2, 2) TD(float, 4, 2) }
  else { TD(double, 2, 3) TD(double, 4, 3) TD(double, 2, 2) TD(double, 4, 2) }
#undef TD
}

}  // namespace

int heat_tune_variant(const adv_heat_desc& d) {
  return (d.dtype == ADV_F64 && d.contract ? 1000 : 0) + d.dtype * 100 + d.order * 10 + d.ndim;
}

// Fraction of a row's lanes that hold grid nodes when rows of nx nodes are cut into tiles bx wide.
static double tile_use(int nx, int bx) { return (double)nx / ((double)((nx + bx - 1) / bx) * bx); }

// rows of 16 lanes (tile 64 wide) where they waste clearly fewer lanes than rows of 32
int heat_row_lanes(int nx) { return tile_use(nx, 64) > tile_use(nx, 128) + 0.02 ? 16 : 32; }

adv_status heat_prepare(const adv_heat_desc& d, const void* u_in, HeatLaunch* L, int rows, int lanes) {
  DeviceInfo di;
  adv_status st = device_info(&di);
  if (st != ADV_OK) return st;
  const int es = d.dtype == ADV_F32 ? 4 : 8;
  const int nz = d.ndim == 3 ? d.nz : 1;
  // TMA needs 16-byte aligned base and strides.
  const bool aligned = ((uintptr_t)u_in % 16 == 0) && (((int64_t)d.nx * es) % 16 == 0) &&
                       (((int64_t)d.nx * d.ny * es) % 16 == 0);
  L->tma = aligned;
  // Four rows per thread (tile 128 x 32): the per-plane bookkeeping of a thread is spread over
  // 16 nodes instead of 8 (FP32 3D O2 with TMA loads).
  const bool rows4_ok = aligned && d.dtype == ADV_F32 && d.order == 2 && d.ndim == 3;
  if (rows == 4 && !rows4_ok) return set_error(ADV_ERR_UNSUPPORTED, "heat: 4 rows per thread need FP32 3D O2 with TMA");
  L->rows = rows == 0 ? (rows4_ok ? 4 : 2) : rows;
  L->warps = L->rows == 4 ? 4 : 8;
  L->lanes = L->rows == 4 ? (lanes != 0 ? lanes : heat_row_lanes(d.nx)) : 32;
  int bx, by, sw, sh, padx, r;
  size_t smem;
  tile_for(d.dtype, d.order, d.ndim, L->rows, L->lanes, &bx, &by, &sw, &sh, &padx, &r, &smem);
  L->block = dim3((unsigned)L->lanes, (unsigned)(32 * L->warps / L->lanes), 1);
  const int tiles_x = (d.nx + bx - 1) / bx, tiles_y = (d.ny + by - 1) / by;
  for (int sk = 0; sk <= 3; ++sk) {
    void* k = pick_kernel(d, L->tma, sk, *L);
    if (!k) return set_error(ADV_ERR_UNSUPPORTED, "heat: no kernel for this configuration");
    ADV_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  void* k0 = pick_kernel(d, L->tma, 1, *L);
  int occ = 0;
  ADV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k0, 32 * L->warps, smem));
  occ = std::max(occ, 1);
  L->occ = occ;
  // One wave: every CTA resident at once, each with an equal share of the (tile, plane) pairs,
  // at least 8 planes each in 3D so the z halo stays small (or what the autotuner picked).
  const int64_t total = (int64_t)tiles_x * tiles_y * nz;
  int64_t min_share = d.ndim == 3 ? 8 : 1;
  const TuneParams tp = tune_lookup(TUNE_HEAT, heat_tune_variant(d), d.nx, d.ny, nz);
  if (tp.set) {
    occ = std::max(1, std::min(occ, tp.a));
    min_share = std::max(1, tp.b);
  }
  const int64_t ctas = std::max<int64_t>(1, std::min<int64_t>((int64_t)di.sms * occ, total / min_share));
  L->tiles_x = tiles_x;
  L->tiles_y = tiles_y;
  L->grid = dim3((unsigned)ctas, 1, 1);
  L->smem = smem;
  std::memset(&L->tmap_in, 0, sizeof(L->tmap_in));
  if (L->tma) {
    EncodeTiledFn enc = encode_tiled_fn();
    if (!enc) return set_error(ADV_ERR_CUDA, "heat: cuTensorMapEncodeTiled unavailable");
    cuuint64_t gdim[3] = {(cuuint64_t)d.nx, (cuuint64_t)d.ny, (cuuint64_t)nz};
    cuuint64_t gstride[2] = {(cuuint64_t)d.nx * es, (cuuint64_t)d.nx * d.ny * es};
    cuuint32_t box[3] = {(cuuint32_t)sw, (cuuint32_t)sh, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    // L2 fetches of 128 bytes: a box row starts one vector before a tile and ends one after it,
    // so 256-byte promotion pulls in up to 480 bytes per row that only a neighbouring tile uses
    // (measured: 256^3 single grid 21.5 -> 21.2 us per launch, the 64-member batch 260 -> 250 us;
    // no promotion measured the same as 128 bytes)
    CUresult cr = enc(&L->tmap_in, d.dtype == ADV_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                      3, const_cast<void*>(u_in), gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return set_error(ADV_ERR_CUDA, "heat: cuTensorMapEncodeTiled failed");
  }
  return ADV_OK;
}

// ------------------------------------------------------------- two Euler steps per launch
void* heat_twostep_kernel_ptr();
size_t heat_twostep_smem();

bool heat2_eligible(const adv_heat_desc& d, const void* u_in) {
  return d.dtype == ADV_F32 && d.ndim == 3 && d.order == 2 && d.nx % 4 == 0 && (uintptr_t)u_in % 16 == 0 &&
         d.nx >= 2 * d.frozen + 1 && d.ny >= 2 * d.frozen + 1 && d.nz >= 2 * d.frozen + 1;
}

adv_status heat2_prepare(const adv_heat_desc& d, const void* u_in, HeatLaunch* L) {
  if (!heat2_eligible(d, u_in)) return set_error(ADV_ERR_UNSUPPORTED, "heat: no two-step kernel for this problem");
  DeviceInfo di;
  adv_status st = device_info(&di);
  if (st != ADV_OK) return st;
  constexpr int BX = 128, BY = 16, SW = 136, SHU = 20;
  void* k = heat_twostep_kernel_ptr();
  const size_t smem = heat_twostep_smem();
  ADV_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  ADV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 128, smem));
  occ = std::max(occ, 1);
  L->tma = true;
  L->occ = occ;
  L->rows = 4;
  L->warps = 4;
  L->lanes = 32;
  L->block = dim3(32, 4, 1);
  L->tiles_x = (d.nx + BX - 1) / BX;
  L->tiles_y = (d.ny + BY - 1) / BY;
  // one wave of CTAs with equal shares of the (tile, plane) pairs, at least 8 planes each
  const int64_t total = (int64_t)L->tiles_x * L->tiles_y * d.nz;
  const int64_t ctas = std::max<int64_t>(1, std::min<int64_t>((int64_t)di.sms * occ, total / 8));
  L->grid = dim3((unsigned)ctas, 1, 1);
  L->smem = smem;
  std::memset(&L->tmap_in, 0, sizeof(L->tmap_in));
  EncodeTiledFn enc = encode_tiled_fn();
  if (!enc) return set_error(ADV_ERR_CUDA, "heat: cuTensorMapEncodeTiled unavailable");
  cuuint64_t gdim[3] = {(cuuint64_t)d.nx, (cuuint64_t)d.ny, (cuuint64_t)d.nz};
  cuuint64_t gstride[2] = {(cuuint64_t)d.nx * 4, (cuuint64_t)d.nx * d.ny * 4};
  cuuint32_t box[3] = {(cuuint32_t)SW, (cuuint32_t)SHU, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult cr = enc(&L->tmap_in, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(u_in), gdim, gstride, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return set_error(ADV_ERR_CUDA, "heat: cuTensorMapEncodeTiled failed");
  return ADV_OK;
}

adv_status heat2_launch(const adv_heat_desc& d, const HeatLaunch& L, const void* u_in, void* u_out, cudaStream_t s) {
  HeatParams<float> p = heat_params<float>(d, L, 1, u_in, u_in, u_out);
  void* args[] = {const_cast<CUtensorMap*>(&L.tmap_in), &p};
  ADV_CUDA_TRY(cudaLaunchKernel(heat_twostep_kernel_ptr(), L.grid, L.block, args, L.smem, s));
  count_launches(1);
  return ADV_OK;
}

template <class T>
static adv_status heat_launch_t(const adv_heat_desc& d, const HeatLaunch& L, int stage, const void* u_in,
                                const void* u_n, void* u_out, cudaStream_t s) {
  HeatParams<T> p = heat_params<T>(d, L, stage, u_in, u_n, u_out);
  const int stage_kind = (stage == 1 && u_n != u_in) ? 0 : stage;
  void* k = pick_kernel(d, L.tma, stage_kind, L);
  void* args[] = {const_cast<CUtensorMap*>(&L.tmap_in), &p};
  ADV_CUDA_TRY(cudaLaunchKernel(k, L.grid, L.block, args, L.smem, s));
  count_launches(1);
  return ADV_OK;
}

void* heat_test_hook_kernel_f32(int lanes);

adv_status heat_launch_test_hook(const adv_heat_desc& d, const HeatLaunch& L, const void* u_in, void* u_out,
                                 cudaStream_t s) {
  if (d.dtype != ADV_F32 || d.ndim != 3 || d.order != 2 || !L.tma || L.rows != 4 || L.warps != 4)
    return set_error(ADV_ERR_UNSUPPORTED, "heat test: the withheld-copy test takes FP32 3D O2 on the TMA path");
  HeatParams<float> p = heat_params<float>(d, L, 1, u_in, u_in, u_out);
  void* k = heat_test_hook_kernel_f32(L.lanes);
  ADV_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
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
