// ensemble.cu -- batched ensembles (adv_ensemble_* in advdiff.h): many independent 3D heat and
// Burgers problems of uneven size advanced by one CUDA graph.
//
// Each member contributes its (tile, z-plane) units to one flat range per kind; a batched stage
// launch cuts that range into equal contiguous shares, one per CTA (two waves of CTAs for heat,
// eight for Burgers), so small members neither leave SMs idle nor pay a launch each
// (heat_batch_kernel, burgers_batch_kernel). The
// device tables hold, per member and per stage slot, the stage parameters and the tensor map of
// the stage input. A run is one graph with two while-nodes that run concurrently: the heat loop
// (a device counter) and the Burgers loop (per-member dt, Lax-Friedrichs constant and stop test,
// the same device code as adv_burgers_run).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "burgers_launch.cuh"
#include "heat_launch.cuh"
#include "nvtx_range.h"

namespace adv {
void* heat_batch_kernel_for(int dtype, int order, bool tma, int stage_kind, int rows, int lanes);
void* heat_batch_mixed_kernel_for(int stage_kind);
template <class T>
void* burgers_batch_kernel_for(const adv_burgers_desc& d);
size_t burgers_smem_f32();
size_t burgers_smem_f64();
}  // namespace adv

using namespace adv;

struct adv_ensemble {
  int device = -1;
  int sms = 0;
  // heat members
  int n_heat = 0, heat_scheme = ADV_EULER, heat_dtype = ADV_F32, heat_order = 2, heat_slots = 0;
  bool heat_tma = true;
  std::vector<adv_heat_member> heat;
  void* heat_tab = nullptr;
  int64_t heat_units = 0;
  int heat_ctas = 0;
  int heat_rows = 2, heat_warps = 8, heat_lanes = 32;  // tile of the batched heat kernel
  // 4-row tiles of two widths (heat_batch_mixed_kernel): the table's first heat_n_wide members
  // (units [0, heat_units_wide)) take rows of 32 lanes and CTAs [0, heat_ctas_wide), the rest
  // rows of 16 lanes
  bool heat_mixed = false;
  int heat_n_wide = 0, heat_ctas_wide = 0;
  int64_t heat_units_wide = 0;
  size_t heat_smem = 0;
  void* heat_k[3] = {nullptr, nullptr, nullptr};
  // Burgers members
  int n_burg = 0, burg_dtype = ADV_F32;
  bool burg_tma = true;
  std::vector<adv_burgers_member> burg;
  void* burg_tab[3] = {nullptr, nullptr, nullptr};
  int64_t burg_units = 0;
  int burg_ctas = 0;
  size_t burg_smem = 0;
  void* burg_k = nullptr;
  BurgersLoopState* states = nullptr;
  std::vector<BurgersLoopState> h_states;
  // loop control (device)
  int64_t* heat_remaining = nullptr;
  int* heat_active = nullptr;
  int* burg_more = nullptr;
  void* dmem = nullptr;
  cudaGraphExec_t graph = nullptr;
};

namespace {

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

size_t elem_bytes(int dtype) { return dtype == ADV_F32 ? 4 : 8; }

// Stage buffers of a heat member: per slot, input, u_n, output and the RK stage number.
struct HeatSlot {
  const void* in;
  const void* un;
  void* out;
  int stage;
};

int heat_slots_of(const adv_heat_member& m, int scheme, HeatSlot* sl) {
  const adv_heat_desc& d = m.desc;
  const size_t one = align256((size_t)d.nx * d.ny * d.nz * elem_bytes(d.dtype));
  char* w1 = static_cast<char*>(m.work);
  char* w2 = w1 + one;
  if (scheme == ADV_EULER) {
    sl[0] = {m.u, m.u, w1, 1};
    sl[1] = {w1, w1, m.u, 1};
    return 2;
  }
  sl[0] = {m.u, m.u, w1, 1};
  sl[1] = {w1, m.u, w2, 2};
  sl[2] = {w2, m.u, m.u, 3};
  return 3;
}

template <class T>
adv_status build_heat_table(adv_ensemble* e, std::vector<unsigned char>& bytes) {
  // Table order: with 4-row tiles each member takes the row width a single grid of its size
  // would (heat_row_lanes), members of 128-wide tiles first; the kernels only see the table, so
  // its order is free.
  std::vector<int> order((size_t)e->n_heat), lanes((size_t)e->n_heat, 32);
  for (int i = 0; i < e->n_heat; ++i) {
    order[(size_t)i] = i;
    if (e->heat_rows == 4) lanes[(size_t)i] = heat_row_lanes(e->heat[(size_t)i].desc.nx);
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return lanes[(size_t)a] > lanes[(size_t)b]; });
  std::vector<HeatBatchInst<T>> tab((size_t)e->n_heat);
  int64_t units = 0, units_wide = 0;
  int n_wide = 0;
  bool tma = true;
  for (int j = 0; j < e->n_heat; ++j) {
    const int i = order[(size_t)j];
    const adv_heat_member& m = e->heat[(size_t)i];
    HeatSlot sl[3];
    const int ns = heat_slots_of(m, e->heat_scheme, sl);
    HeatLaunch L;
    for (int s = 0; s < ns; ++s) {
      adv_status st = heat_prepare(m.desc, sl[s].in, &L, e->heat_rows, lanes[(size_t)i]);  // the batched tile
      if (st != ADV_OK) return st;
      tma = tma && L.tma;
      tab[(size_t)j].tmap[s] = L.tmap_in;
      tab[(size_t)j].p[s] = heat_params<T>(m.desc, L, sl[s].stage, sl[s].in, sl[s].un, sl[s].out);
    }
    tab[(size_t)j].unit_begin = units;
    units += (int64_t)L.tiles_x * L.tiles_y * m.desc.nz;
    if (lanes[(size_t)i] == 32) {
      ++n_wide;
      units_wide = units;
    }
    e->heat_smem = L.smem;
  }
  e->heat_tma = tma;
  e->heat_units = units;
  e->heat_n_wide = n_wide;
  e->heat_units_wide = units_wide;
  e->heat_mixed = n_wide > 0 && n_wide < e->n_heat;
  e->heat_lanes = n_wide > 0 ? 32 : 16;
  bytes.resize(tab.size() * sizeof(HeatBatchInst<T>));
  std::memcpy(bytes.data(), tab.data(), bytes.size());
  return ADV_OK;
}

template <class T>
adv_status build_burgers_tables(adv_ensemble* e, std::vector<unsigned char> (&bytes)[3]) {
  using K = typename KeyOf<T>::type;
  std::vector<BurgersBatchInst<T>> tab[3];
  for (auto& t : tab) t.resize((size_t)e->n_burg);
  int64_t units = 0;
  bool tma = true;
  for (int i = 0; i < e->n_burg; ++i) {
    const adv_burgers_member& m = e->burg[i];
    const adv_burgers_desc& d = m.desc;
    const size_t one = align256((size_t)d.nx * d.ny * d.nz * sizeof(T));
    char* w1 = static_cast<char*>(m.work);
    char* w2 = w1 + one;
    BurgersLoopState* st = e->states + i;
    K* keys = sizeof(T) == 4 ? reinterpret_cast<K*>(st->maxbits) : reinterpret_cast<K*>(st->maxbits64);
    BurgersStageArgs a[3] = {};
    for (auto& x : a) {
      x.dt_dev = &st->dt;
      x.active = &st->active;
      x.u_n = m.u;
    }
    a[0].stage = 1; a[0].u_in = m.u; a[0].u_out = w1; a[0].alpha_dev = &st->alpha0; a[0].maxabs_key = keys + 1;
    a[1].stage = 2; a[1].u_in = w1; a[1].u_out = w2; a[1].alpha_key = keys + 1; a[1].maxabs_key = keys + 2;
    a[2].stage = 3; a[2].u_in = w2; a[2].u_out = m.u; a[2].alpha_key = keys + 2; a[2].maxabs_key = keys + 0;
    BurgersLaunch L;
    for (int s = 0; s < 3; ++s) {
      adv_status r = burgers_prepare(d, a[s].u_in, &L);
      if (r != ADV_OK) return r;
      tma = tma && L.tma;
      tab[s][i].tmap = L.tmap_in;
      tab[s][i].p = burgers_params<T>(d, L, a[s]);
    }
    for (int s = 0; s < 3; ++s) tab[s][i].unit_begin = units;
    units += (int64_t)L.tiles_x * L.tiles_y * d.nz;
  }
  // One load path for the whole batch: the pipeline's slot parities assume it.
  if (!tma)
    for (auto& t : tab)
      for (auto& x : t) x.p.tma = 0;
  e->burg_tma = tma;
  e->burg_units = units;
  for (int s = 0; s < 3; ++s) {
    bytes[s].resize(tab[s].size() * sizeof(BurgersBatchInst<T>));
    std::memcpy(bytes[s].data(), tab[s].data(), bytes[s].size());
  }
  return ADV_OK;
}

int one_wave_ctas(void* kernel, int threads, size_t smem, int sms, int64_t units, adv_status* st) {
  int occ = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem);
  if (e != cudaSuccess) {
    *st = cuda_error(e, "ensemble: occupancy");
    return 0;
  }
  occ = std::max(occ, 1);
  // at least 8 planes per CTA so the z halo stays small
  return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * occ, units / 8));
}

adv_status launch_heat_slot(adv_ensemble* e, int slot, const int* active, cudaStream_t s) {
  const void* tab = e->heat_tab;
  int n = e->n_heat;
  int64_t units = e->heat_units;
  if (e->heat_mixed) {
    int n_wide = e->heat_n_wide, ctas_wide = e->heat_ctas_wide;
    int64_t units_wide = e->heat_units_wide;
    void* args[] = {&tab, &n_wide, &n, &units_wide, &units, &ctas_wide, &slot, &active};
    ADV_CUDA_TRY(cudaLaunchKernel(e->heat_k[slot], dim3((unsigned)e->heat_ctas), dim3(128, 1, 1), args, e->heat_smem,
                                  s));
  } else {
    void* args[] = {&tab, &n, &units, &slot, &active};
    const dim3 block((unsigned)e->heat_lanes, (unsigned)(32 * e->heat_warps / e->heat_lanes), 1);
    ADV_CUDA_TRY(cudaLaunchKernel(e->heat_k[slot], dim3((unsigned)e->heat_ctas), block, args, e->heat_smem, s));
  }
  count_launches(1);
  return ADV_OK;
}

adv_status launch_burgers_stage(adv_ensemble* e, int stage, cudaStream_t s) {
  const void* tab = e->burg_tab[stage - 1];
  int n = e->n_burg;
  int64_t units = e->burg_units;
  int tma = e->burg_tma ? 1 : 0;
  void* args[] = {&tab, &n, &units, &tma};
  ADV_CUDA_TRY(cudaLaunchKernel(e->burg_k, dim3((unsigned)e->burg_ctas), dim3(256, 1, 1), args, e->burg_smem, s));
  count_launches(1);
  return ADV_OK;
}

// One iteration of the heat loop: a pair of Euler steps (slots 0, 1) or one SSP-RK3 step.
adv_status heat_body(adv_ensemble* e, unsigned long long cond, int use_cond, cudaStream_t s) {
  adv_status st = loop_tick(e->heat_remaining, e->heat_active, cond, use_cond, s);
  for (int k = 0; st == ADV_OK && k < e->heat_slots; ++k) st = launch_heat_slot(e, k, e->heat_active, s);
  return st;
}

// One step of every Burgers member (predicated per member on the device).
adv_status burgers_body(adv_ensemble* e, unsigned long long cond, int use_cond, cudaStream_t s) {
  adv_status st = burgers_loop_begin_step_batch(e->states, e->n_burg, e->burg_dtype, cond, use_cond, e->burg_more, s);
  for (int k = 1; st == ADV_OK && k <= 3; ++k) st = launch_burgers_stage(e, k, s);
  return st;
}

// The run graph: a while-node per kind, no edge between them, so the two loops run concurrently.
adv_status build_graph(adv_ensemble* e) {
  cudaGraph_t g = nullptr;
  ADV_CUDA_TRY(cudaGraphCreate(&g, 0));
  cudaStream_t cs = nullptr;
  cudaError_t err = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  adv_status st = err == cudaSuccess ? ADV_OK : cuda_error(err, "ensemble: capture stream");
  const int64_t launches_before = adv_kernel_launch_count();
  for (int kind = 0; kind < 2 && st == ADV_OK; ++kind) {
    if ((kind == 0 ? e->n_heat : e->n_burg) == 0) continue;
    cudaGraphConditionalHandle h = 0;
    err = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (err == cudaSuccess) err = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
    if (err == cudaSuccess)
      err = cudaStreamBeginCaptureToGraph(cs, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
    if (err != cudaSuccess) {
      st = cuda_error(err, "ensemble: while-node");
      break;
    }
    st = kind == 0 ? heat_body(e, (unsigned long long)h, 1, cs) : burgers_body(e, (unsigned long long)h, 1, cs);
    cudaGraph_t body = nullptr;
    err = cudaStreamEndCapture(cs, &body);
    if (st == ADV_OK && err != cudaSuccess) st = cuda_error(err, "ensemble: capture");
  }
  count_launches(launches_before - adv_kernel_launch_count());  // captured, not launched
  if (st == ADV_OK) {
    err = cudaGraphInstantiate(&e->graph, g, 0);
    if (err != cudaSuccess) {
      e->graph = nullptr;
      st = cuda_error(err, "ensemble: instantiate");
    }
  }
  if (cs) cudaStreamDestroy(cs);
  cudaGraphDestroy(g);
  return st;
}

adv_status check_device(const adv_ensemble* e) {
  int dev = -1;
  ADV_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != e->device) return set_error(ADV_ERR_INVALID_ARG, "ensemble: plan belongs to another device");
  return ADV_OK;
}

adv_status create_impl(const adv_heat_member* heat, int n_heat, int scheme, const adv_burgers_member* burgers,
                       int n_burgers, adv_ensemble* e) {
  if (n_heat < 0 || n_burgers < 0 || (n_heat > 0 && !heat) || (n_burgers > 0 && !burgers))
    return set_error(ADV_ERR_INVALID_ARG, "ensemble: bad member arrays");
  if (n_heat + n_burgers == 0) return set_error(ADV_ERR_INVALID_ARG, "ensemble: no members");
  if (scheme != ADV_EULER && scheme != ADV_SSPRK3) return set_error(ADV_ERR_INVALID_ARG, "ensemble: bad heat time scheme");
  DeviceInfo di;
  adv_status st = device_info(&di);
  if (st != ADV_OK) return st;
  e->device = di.device;
  e->sms = di.sms;
  e->heat_scheme = scheme;
  e->heat_slots = scheme == ADV_EULER ? 2 : 3;
  e->n_heat = n_heat;
  e->n_burg = n_burgers;
  e->heat.assign(heat, heat + n_heat);
  e->burg.assign(burgers, burgers + n_burgers);
  for (int i = 0; i < n_heat; ++i) {
    const adv_heat_member& m = heat[i];
    if ((st = heat_validate(&m.desc)) != ADV_OK) return st;
    if (m.desc.ndim != 3) return set_error(ADV_ERR_INVALID_ARG, "ensemble: heat members must be 3D");
    if (!m.u || !m.work) return set_error(ADV_ERR_INVALID_ARG, "ensemble: null heat buffer");
    if (m.desc.dtype != heat[0].desc.dtype || m.desc.order != heat[0].desc.order)
      return set_error(ADV_ERR_INVALID_ARG, "ensemble: heat members must share dtype and order");
    if (m.desc.dtype == ADV_F64 && m.desc.contract)
      return set_error(ADV_ERR_UNSUPPORTED, "ensemble: FP64 heat members take the reference's rounding (contract 0)");
  }
  for (int i = 0; i < n_burgers; ++i) {
    const adv_burgers_member& m = burgers[i];
    const adv_burgers_desc& d = m.desc;
    const adv_burgers_desc& d0 = burgers[0].desc;
    if ((st = burgers_validate(&d)) != ADV_OK) return st;
    if (!m.u || !m.work) return set_error(ADV_ERR_INVALID_ARG, "ensemble: null Burgers buffer");
    const bool visc = d.kx != 0.0 || d.ky != 0.0 || d.kz != 0.0;
    const bool visc0 = d0.kx != 0.0 || d0.ky != 0.0 || d0.kz != 0.0;
    const bool div_differs = d.dtype == ADV_F32 ? d.div != d0.div : (d.div == ADV_DIV_FAST) != (d0.div == ADV_DIV_FAST);
    if (d.dtype != d0.dtype || d.weno != d0.weno || visc != visc0 || div_differs)
      return set_error(ADV_ERR_INVALID_ARG, "ensemble: Burgers members must share dtype, weno, div and viscosity");
    if (m.dt_rule != ADV_DT_FIXED && m.dt_rule != ADV_DT_MAXU)
      return set_error(ADV_ERR_INVALID_ARG, "ensemble: bad Burgers dt rule");
    if (!(m.cfl > 0) || !std::isfinite(m.tEnd) || m.max_steps < 0)
      return set_error(ADV_ERR_INVALID_ARG, "ensemble: bad Burgers cfl/tEnd/max_steps");
  }
  if (n_heat > 0) {
    e->heat_dtype = heat[0].desc.dtype;
    e->heat_order = heat[0].desc.order;
  }
  if (n_burgers > 0) e->burg_dtype = burgers[0].desc.dtype;

  // device block: heat table | Burgers tables x3 | loop states | control words
  const size_t heat_tab_bytes = align256((size_t)n_heat * (e->heat_dtype == ADV_F32 ? sizeof(HeatBatchInst<float>)
                                                                                      : sizeof(HeatBatchInst<double>)));
  const size_t burg_tab_bytes = align256((size_t)n_burgers * (e->burg_dtype == ADV_F32 ? sizeof(BurgersBatchInst<float>)
                                                                                          : sizeof(BurgersBatchInst<double>)));
  const size_t states_bytes = align256((size_t)n_burgers * sizeof(BurgersLoopState));
  const size_t total = heat_tab_bytes + 3 * burg_tab_bytes + states_bytes + 256;
  cudaError_t err = cudaMalloc(&e->dmem, total);
  if (err != cudaSuccess) {
    e->dmem = nullptr;
    cudaGetLastError();
    return set_error(ADV_ERR_ALLOC, "ensemble: device tables");
  }
  char* base = static_cast<char*>(e->dmem);
  e->heat_tab = base;
  for (int s = 0; s < 3; ++s) e->burg_tab[s] = base + heat_tab_bytes + s * burg_tab_bytes;
  e->states = reinterpret_cast<BurgersLoopState*>(base + heat_tab_bytes + 3 * burg_tab_bytes);
  char* ctl = base + heat_tab_bytes + 3 * burg_tab_bytes + states_bytes;
  e->heat_remaining = reinterpret_cast<int64_t*>(ctl);
  e->heat_active = reinterpret_cast<int*>(ctl + 8);
  e->burg_more = reinterpret_cast<int*>(ctl + 16);
  ADV_CUDA_TRY(cudaMemset(ctl, 0, 256));

  if (n_heat > 0) {
    std::vector<unsigned char> bytes;
    // the 4-row tile when every member's stage takes it (FP32 O2 with TMA loads; rows of 32 or 16
    // lanes per member), else 2 rows of 32 lanes.
    e->heat_rows = 4;
    e->heat_warps = 4;
    e->heat_lanes = 32;
    st = e->heat_dtype == ADV_F32 ? build_heat_table<float>(e, bytes) : ADV_ERR_UNSUPPORTED;
    if (st == ADV_ERR_UNSUPPORTED) {
      e->heat_rows = 2;
      e->heat_warps = 8;
      e->heat_lanes = 32;
      bytes.clear();
      st = e->heat_dtype == ADV_F32 ? build_heat_table<float>(e, bytes) : build_heat_table<double>(e, bytes);
    }
    if (st != ADV_OK) return st;
    ADV_CUDA_TRY(cudaMemcpy(e->heat_tab, bytes.data(), bytes.size(), cudaMemcpyHostToDevice));
    for (int k = 0; k < e->heat_slots; ++k) {
      const int sk = scheme == ADV_EULER ? 1 : k + 1;
      e->heat_k[k] = e->heat_mixed ? heat_batch_mixed_kernel_for(sk)
                                   : heat_batch_kernel_for(e->heat_dtype, e->heat_order, e->heat_tma, sk, e->heat_rows,
                                                           e->heat_lanes);
      if (!e->heat_k[k]) return set_error(ADV_ERR_UNSUPPORTED, "ensemble: no batched heat kernel");
      ADV_CUDA_TRY(cudaFuncSetAttribute(e->heat_k[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->heat_smem));
    }
    e->heat_ctas = one_wave_ctas(e->heat_k[0], 32 * e->heat_warps, e->heat_smem, e->sms, e->heat_units, &st);
    if (st != ADV_OK) return st;
    // two waves of equal shares instead of one: CTAs whose segments finish early leave their SM
    // to the second wave (measured 2-6% faster on the mixed-size ensemble)
    e->heat_ctas = (int)std::max<int64_t>(1, std::min<int64_t>(2 * (int64_t)e->heat_ctas, e->heat_units / 4));
    if (e->heat_mixed) {
      // CTAs per width group in proportion to its units (a unit costs the same in both), at
      // least one each
      e->heat_ctas = std::max(e->heat_ctas, 2);
      const double f = (double)e->heat_units_wide / (double)e->heat_units;
      e->heat_ctas_wide = std::min(e->heat_ctas - 1, std::max(1, (int)std::lround(f * e->heat_ctas)));
    }
  }
  if (n_burgers > 0) {
    std::vector<unsigned char> bytes[3];
    st = e->burg_dtype == ADV_F32 ? build_burgers_tables<float>(e, bytes) : build_burgers_tables<double>(e, bytes);
    if (st != ADV_OK) return st;
    for (int s = 0; s < 3; ++s)
      ADV_CUDA_TRY(cudaMemcpy(e->burg_tab[s], bytes[s].data(), bytes[s].size(), cudaMemcpyHostToDevice));
    e->burg_k = e->burg_dtype == ADV_F32 ? burgers_batch_kernel_for<float>(burgers[0].desc)
                                         : burgers_batch_kernel_for<double>(burgers[0].desc);
    if (!e->burg_k) return set_error(ADV_ERR_UNSUPPORTED, "ensemble: no batched Burgers kernel");
    e->burg_smem = e->burg_dtype == ADV_F32 ? burgers_smem_f32() : burgers_smem_f64();
    ADV_CUDA_TRY(cudaFuncSetAttribute(e->burg_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->burg_smem));
    e->burg_ctas = one_wave_ctas(e->burg_k, 256, e->burg_smem, e->sms, e->burg_units, &st);
    if (st != ADV_OK) return st;
    // eight waves of equal shares: the batched WENO stage's per-pair cost varies across members
    // and segments, and later waves balance it (measured on the 32-member Burgers batch: 198 ms
    // per 30 steps with one wave, 177 with four, 169 with eight, 170 with sixteen)
    e->burg_ctas = (int)std::max<int64_t>(1, std::min<int64_t>(8 * (int64_t)e->burg_ctas, e->burg_units / 4));
    e->h_states.resize((size_t)n_burgers);
  }
  return ADV_OK;
}

void destroy_impl(adv_ensemble* e) {
  if (e->graph) cudaGraphExecDestroy(e->graph);
  if (e->dmem) cudaFree(e->dmem);
  delete e;
}

}  // namespace

extern "C" {

adv_status adv_ensemble_create(const adv_heat_member* heat, int n_heat, int heat_time_scheme,
                               const adv_burgers_member* burgers, int n_burgers, adv_ensemble** out) {
  ADV_NVTX_RANGE("adv_ensemble_create");
  if (!out) return set_error(ADV_ERR_INVALID_ARG, "ensemble: null output");
  *out = nullptr;
  adv_ensemble* e = new (std::nothrow) adv_ensemble();
  if (!e) return set_error(ADV_ERR_ALLOC, "ensemble: host plan");
  const adv_status st = create_impl(heat, n_heat, heat_time_scheme, burgers, n_burgers, e);
  if (st != ADV_OK) {
    destroy_impl(e);
    return st;
  }
  *out = e;
  return ADV_OK;
}

adv_status adv_ensemble_run(adv_ensemble* e, int64_t heat_steps, int flags, void* stream) {
  ADV_NVTX_RANGE("adv_ensemble_run");
  if (!e) return set_error(ADV_ERR_INVALID_ARG, "ensemble: null plan");
  if (heat_steps < 0) return set_error(ADV_ERR_INVALID_ARG, "ensemble: negative heat step count");
  if (flags & ~ADV_ENSEMBLE_DIRECT) return set_error(ADV_ERR_INVALID_ARG, "ensemble: unknown flags");
  adv_status st = check_device(e);
  if (st != ADV_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if ((st = reject_capture(s, "ensemble run")) != ADV_OK) return st;
  const int64_t heat_iters = e->n_heat == 0 ? 0 : (e->heat_scheme == ADV_EULER ? heat_steps / 2 : heat_steps);

  // Burgers loop states: t = 0, then max|u^0| of every member into its slot-0 key.
  for (int i = 0; i < e->n_burg; ++i) {
    const adv_burgers_member& m = e->burg[i];
    e->h_states[i] = burgers_loop_state(m.desc, m.tEnd, m.cfl, m.dt_rule, m.C, m.max_steps);
  }
  if (e->n_burg > 0) {
    ADV_CUDA_TRY(cudaMemcpyAsync(e->states, e->h_states.data(), e->h_states.size() * sizeof(BurgersLoopState),
                                 cudaMemcpyHostToDevice, s));
    for (int i = 0; i < e->n_burg; ++i) {
      const adv_burgers_desc& d = e->burg[i].desc;
      void* key0 = e->burg_dtype == ADV_F32 ? (void*)&e->states[i].maxbits[0] : (void*)&e->states[i].maxbits64[0];
      if ((st = max_abs_launch(e->burg_dtype, e->burg[i].u, (int64_t)d.nx * d.ny * d.nz, key0, s)) != ADV_OK) return st;
    }
  }
  ADV_CUDA_TRY(cudaMemcpyAsync(e->heat_remaining, &heat_iters, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  ADV_CUDA_TRY(cudaStreamSynchronize(s));  // the host sources above are locals / plan fields

  if (flags & ADV_ENSEMBLE_DIRECT) {
    for (int64_t it = 0; it < heat_iters; ++it)
      for (int k = 0; k < e->heat_slots; ++k)
        if ((st = launch_heat_slot(e, k, nullptr, s)) != ADV_OK) return st;
    if (e->n_burg > 0) {
      for (;;) {
        for (int c = 0; c < 8; ++c)
          if ((st = burgers_body(e, 0, 0, s)) != ADV_OK) return st;
        int more = 0;
        ADV_CUDA_TRY(cudaMemcpyAsync(&more, e->burg_more, sizeof(int), cudaMemcpyDeviceToHost, s));
        ADV_CUDA_TRY(cudaStreamSynchronize(s));
        if (!more) break;
      }
    }
  } else {
    if (!e->graph && (st = build_graph(e)) != ADV_OK) return st;
    ADV_CUDA_TRY(cudaGraphLaunch(e->graph, s));
    if (e->n_heat > 0) count_launches(std::max<int64_t>(heat_iters, 1) * (1 + e->heat_slots));
  }
  // An odd Euler step count ends with one more step into w1, copied back to u.
  if (e->n_heat > 0 && e->heat_scheme == ADV_EULER && heat_steps % 2) {
    if ((st = launch_heat_slot(e, 0, nullptr, s)) != ADV_OK) return st;
    for (int i = 0; i < e->n_heat; ++i) {
      const adv_heat_desc& d = e->heat[i].desc;
      ADV_CUDA_TRY(cudaMemcpyAsync(e->heat[i].u, e->heat[i].work, (size_t)d.nx * d.ny * d.nz * elem_bytes(d.dtype),
                                   cudaMemcpyDeviceToDevice, s));
    }
  }
  if (e->n_burg > 0) {
    ADV_CUDA_TRY(cudaMemcpyAsync(e->h_states.data(), e->states, e->h_states.size() * sizeof(BurgersLoopState),
                                 cudaMemcpyDeviceToHost, s));
  }
  ADV_CUDA_TRY(cudaStreamSynchronize(s));
  if (!(flags & ADV_ENSEMBLE_DIRECT) && e->n_burg > 0) {
    int64_t iters = 1;
    for (const auto& h : e->h_states) iters = std::max<int64_t>(iters, h.step);
    count_launches(4 * iters);
  }
  return read_and_clear_device_status(s);
}

adv_status adv_ensemble_burgers_result(const adv_ensemble* e, int i, double* t, int64_t* steps) {
  if (!e || i < 0 || i >= e->n_burg) return set_error(ADV_ERR_INVALID_ARG, "ensemble: bad Burgers member index");
  if (t) *t = e->h_states[i].t;
  if (steps) *steps = e->h_states[i].step;
  return ADV_OK;
}

adv_status adv_ensemble_shape(const adv_ensemble* e, int64_t* heat_units, int* heat_ctas, int64_t* burgers_units,
                              int* burgers_ctas) {
  if (!e) return set_error(ADV_ERR_INVALID_ARG, "ensemble: null plan");
  if (heat_units) *heat_units = e->heat_units;
  if (heat_ctas) *heat_ctas = e->heat_ctas;
  if (burgers_units) *burgers_units = e->burg_units;
  if (burgers_ctas) *burgers_ctas = e->burg_ctas;
  return ADV_OK;
}

adv_status adv_ensemble_destroy(adv_ensemble* e) {
  if (!e) return ADV_OK;
  const int dev = e->device;
  int prev = -1;
  cudaGetDevice(&prev);
  if (dev >= 0 && prev != dev) cudaSetDevice(dev);
  destroy_impl(e);
  if (prev >= 0 && dev >= 0 && prev != dev) cudaSetDevice(prev);
  return ADV_OK;
}

}  // extern "C"
