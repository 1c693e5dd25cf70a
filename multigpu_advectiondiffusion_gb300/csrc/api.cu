// api.cu -- the native C ABI (include/advdiff.h): validation, launch preparation, CUDA-graph
// time loops, seeded initial conditions and the result.bin writer.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "adv_device.cuh"
#include "adv_internal.h"
#include "nvtx_range.h"

namespace adv {

adv_status burgers_launch_f32(const adv_burgers_desc& d, const BurgersLaunch& L, const BurgersStageArgs& a,
                              cudaStream_t s);
adv_status burgers_launch_f64(const adv_burgers_desc& d, const BurgersLaunch& L, const BurgersStageArgs& a,
                              cudaStream_t s);
size_t burgers_smem_f32();
size_t burgers_smem_f64();
template <class T>
void* burgers_kernel_for(const adv_burgers_desc& d);

// ---------------------------------------------------------------------------- errors
static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches{0};

adv_status set_error(adv_status s, const std::string& msg) {
  g_last_error = msg;
  return s;
}
adv_status cuda_error(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return ADV_ERR_CUDA;
}
void count_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// ---------------------------------------------------------------------- device info
adv_status device_info(DeviceInfo* out) {
  static std::mutex mu;
  static DeviceInfo cache[64];
  int dev = 0;
  ADV_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(ADV_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(mu);
  if (cache[dev].device != dev) {
    cudaDeviceProp prop;
    ADV_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
    cache[dev].device = dev;
    cache[dev].sms = prop.multiProcessorCount;
    cache[dev].cc_major = prop.major;
    cache[dev].cc_minor = prop.minor;
    cache[dev].smem_optin = prop.sharedMemPerBlockOptin;
  }
  *out = cache[dev];
  return ADV_OK;
}

EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// ------------------------------------------------------------------------ Burgers prep
adv_status burgers_validate(const adv_burgers_desc* d) {
  if (!d) return set_error(ADV_ERR_INVALID_ARG, "burgers: null descriptor");
  if (d->dtype != ADV_F32 && d->dtype != ADV_F64) return set_error(ADV_ERR_INVALID_ARG, "burgers: bad dtype");
  if (d->weno != ADV_WENO5_JS && d->weno != ADV_WENO5_Z) return set_error(ADV_ERR_INVALID_ARG, "burgers: bad weno");
  if (d->lf != ADV_LF_LOCAL && d->lf != ADV_LF_GLOBAL) return set_error(ADV_ERR_INVALID_ARG, "burgers: bad lf");
  if (d->bc != ADV_BC_FROZEN && d->bc != ADV_BC_PERIODIC) return set_error(ADV_ERR_INVALID_ARG, "burgers: bad bc");
  if (d->div != ADV_DIV_F32 && d->div != ADV_DIV_F64 && d->div != ADV_DIV_FAST)
    return set_error(ADV_ERR_INVALID_ARG, "burgers: bad div");
  if (d->nx < 1 || d->ny < 1 || d->nz < 1) return set_error(ADV_ERR_INVALID_ARG, "burgers: empty grid");
  if (d->nx > (1 << 30) || d->ny > (1 << 30) || d->nz > (1 << 30))
    return set_error(ADV_ERR_INVALID_ARG, "burgers: dimension too large");
  const bool twod = d->nz == 1;  // a 2D problem: one plane, no z fluxes
  if (d->bc == ADV_BC_PERIODIC && (d->nx < 6 || d->ny < 6 || (!twod && d->nz < 6)))
    return set_error(ADV_ERR_INVALID_ARG, "burgers: periodic grids need at least 6 cells per axis");
  if (twod && d->kz != 0.0) return set_error(ADV_ERR_INVALID_ARG, "burgers: a 2D grid (nz == 1) takes kz = 0");
  if (!(d->dx > 0) || !(d->dy > 0) || !(d->dz > 0)) return set_error(ADV_ERR_INVALID_ARG, "burgers: spacing must be > 0");
  return ADV_OK;
}

int burgers_tune_variant(const adv_burgers_desc& d) {
  const int visc = (d.kx != 0.0 || d.ky != 0.0 || d.kz != 0.0) ? 1 : 0;
  return d.dtype * 1000 + d.weno * 100 + d.div * 10 + visc;
}

adv_status burgers_prepare(const adv_burgers_desc& d, const void* u_in, BurgersLaunch* L) {
  DeviceInfo di;
  adv_status st = device_info(&di);
  if (st != ADV_OK) return st;
  const int es = d.dtype == ADV_F32 ? 4 : 8;
  const bool aligned = ((uintptr_t)u_in % 16 == 0) && (((int64_t)d.nx * es) % 16 == 0) &&
                       (((int64_t)d.nx * d.ny * es) % 16 == 0);
  L->tma = aligned;
  L->block = dim3(256, 1, 1);
  const int tiles_x = (d.nx + 31) / 32, tiles_y = (d.ny + 15) / 16;
  L->smem = d.dtype == ADV_F32 ? burgers_smem_f32() : burgers_smem_f64();
  void* k = d.dtype == ADV_F32 ? burgers_kernel_for<float>(d) : burgers_kernel_for<double>(d);
  if (!k) return set_error(ADV_ERR_UNSUPPORTED, "burgers: no kernel for this configuration");
  ADV_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L->smem));
  int occ = 0;
  ADV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 256, L->smem));
  occ = std::max(occ, 1);
  L->occ = occ;
  // CTAs with equal shares of the (tile, plane) pairs (at least 8 planes, or
  // what the autotuner picked).
  const int64_t total = (int64_t)tiles_x * tiles_y * d.nz;
  int64_t min_share = 8;
  const TuneParams tp = tune_lookup(TUNE_BURGERS, burgers_tune_variant(d), d.nx, d.ny, d.nz);
  if (tp.set) {
    occ = std::max(1, std::min(occ, tp.a));
    min_share = std::max(1, tp.b);
  }
  // four waves of CTAs rather than one: the cost of a (tile, plane) pair varies (edge tiles patch
  // their halo, segments restart the pipeline), and later waves fill the SMs whose CTAs finished
  // early (measured at 256^3: 456 us per stage with one wave, 403 with four, 414 with eight)
  const int64_t ctas = std::max<int64_t>(1, std::min<int64_t>(4 * (int64_t)di.sms * occ, total / min_share));
  L->tiles_x = tiles_x;
  L->tiles_y = tiles_y;
  L->grid = dim3((unsigned)ctas, 1, 1);
  std::memset(&L->tmap_in, 0, sizeof(L->tmap_in));
  if (L->tma) {
    EncodeTiledFn enc = encode_tiled_fn();
    if (!enc) return set_error(ADV_ERR_CUDA, "burgers: cuTensorMapEncodeTiled unavailable");
    cuuint64_t gdim[3] = {(cuuint64_t)d.nx, (cuuint64_t)d.ny, (cuuint64_t)d.nz};
    cuuint64_t gstride[2] = {(cuuint64_t)d.nx * es, (cuuint64_t)d.nx * d.ny * es};
    cuuint32_t box[3] = {40, 22, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult cr = enc(&L->tmap_in, d.dtype == ADV_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                      3, const_cast<void*>(u_in), gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return set_error(ADV_ERR_CUDA, "burgers: cuTensorMapEncodeTiled failed");
  }
  return ADV_OK;
}

adv_status burgers_launch(const adv_burgers_desc& d, const BurgersLaunch& L, const BurgersStageArgs& a,
                          cudaStream_t s) {
  if (a.stage < 1 || a.stage > 3) return set_error(ADV_ERR_INVALID_ARG, "burgers: stage must be 1, 2 or 3");
  return d.dtype == ADV_F32 ? burgers_launch_f32(d, L, a, s) : burgers_launch_f64(d, L, a, s);
}

bool stream_capturing(cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) return false;
  return cs != cudaStreamCaptureStatusNone;
}

adv_status reject_capture(cudaStream_t s, const char* what) {
  if (!stream_capturing(s)) return ADV_OK;
  return set_error(ADV_ERR_UNSUPPORTED, std::string(what) +
                                            ": reads its results back to the host, so it cannot be recorded into a "
                                            "stream capture (capture the stage calls instead)");
}

// Instantiated CUDA graphs of the run loops, keyed by everything the captured launches depend
// on (device, descriptor, buffer addresses, chunk length). A repeated run on the same buffers
// replays the cached graph with no capture or instantiation cost. At most 32 entries (LRU).
class GraphCache {
 public:
  cudaGraphExec_t get(const std::string& key) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = m_.find(key);
    if (it == m_.end()) return nullptr;
    it->second.second = ++tick_;
    return it->second.first;
  }
  void put(const std::string& key, cudaGraphExec_t e) {
    std::lock_guard<std::mutex> lk(mu_);
    if (m_.size() >= 32) {
      auto old = m_.begin();
      for (auto it = m_.begin(); it != m_.end(); ++it)
        if (it->second.second < old->second.second) old = it;
      cudaDeviceSynchronize();  // the evicted graph may still be running
      cudaGraphExecDestroy(old->second.first);
      m_.erase(old);
    }
    m_[key] = {e, ++tick_};
  }
  void clear() {
    std::lock_guard<std::mutex> lk(mu_);
    if (m_.empty()) return;
    cudaDeviceSynchronize();  // a cached graph may still be running
    for (auto& kv : m_) cudaGraphExecDestroy(kv.second.first);
    m_.clear();
  }

 private:
  std::mutex mu_;
  std::map<std::string, std::pair<cudaGraphExec_t, uint64_t>> m_;
  uint64_t tick_ = 0;
};
static GraphCache g_graphs;
void graph_cache_clear() { g_graphs.clear(); }

template <class... A>
static std::string graph_key(const char* tag, const A&... parts) {
  int dev = -1;
  cudaGetDevice(&dev);
  std::string k(tag);
  k.append(reinterpret_cast<const char*>(&dev), sizeof dev);
  (k.append(reinterpret_cast<const char*>(&parts), sizeof(parts)), ...);
  return k;
}

// Runs `body` (which enqueues one chunk of work on a stream) `reps` times: captured once into a
// CUDA graph (cached under `key`) and replayed, unless the caller's stream is itself being
// captured, in which case the launches go straight into the caller's capture.
template <class F>
static adv_status replay(const std::string& key, cudaStream_t s, int64_t reps, F body, int64_t launches_per_call) {
  if (reps <= 0) return ADV_OK;
  if (stream_capturing(s)) {
    for (int64_t r = 0; r < reps; ++r) {
      adv_status st = body(s);
      if (st != ADV_OK) return st;
    }
    return ADV_OK;
  }
  cudaGraphExec_t ge = g_graphs.get(key);
  if (!ge) {
    cudaStream_t cs;
    ADV_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    adv_status st = ADV_OK;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      const int64_t before = g_launches.load();
      st = body(cs);
      g_launches.store(before);  // launches are counted on replay
      e = cudaStreamEndCapture(cs, &g);
    }
    if (e == cudaSuccess && st == ADV_OK) e = cudaGraphInstantiate(&ge, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (st != ADV_OK) return st;
    if (e != cudaSuccess) return cuda_error(e, "graph capture");
    g_graphs.put(key, ge);
  }
  for (int64_t r = 0; r < reps; ++r) {
    cudaError_t e = cudaGraphLaunch(ge, s);
    if (e != cudaSuccess) return cuda_error(e, "graph replay");
    count_launches(launches_per_call);
  }
  return ADV_OK;
}

}  // namespace adv

using namespace adv;

extern "C" {

const char* adv_last_error_string(void) { return g_last_error.c_str(); }
int adv_abi_version(void) { return ADV_ABI_VERSION; }
int64_t adv_kernel_launch_count(void) { return g_launches.load(); }

int adv_bounds_checked(void) {
#ifdef ADV_BOUNDS_CHECK
  return 1;
#else
  return 0;
#endif
}

const char* adv_status_string(adv_status s) {
  switch (s) {
    case ADV_OK: return "ADV_OK";
    case ADV_ERR_INVALID_ARG: return "ADV_ERR_INVALID_ARG";
    case ADV_ERR_CUDA: return "ADV_ERR_CUDA";
    case ADV_ERR_TIMEOUT: return "ADV_ERR_TIMEOUT";
    case ADV_ERR_NONFINITE: return "ADV_ERR_NONFINITE";
    case ADV_ERR_CFL: return "ADV_ERR_CFL";
    case ADV_ERR_UNSUPPORTED: return "ADV_ERR_UNSUPPORTED";
    case ADV_ERR_ALLOC: return "ADV_ERR_ALLOC";
    case ADV_ERR_BOUNDS: return "ADV_ERR_BOUNDS";
  }
  return "ADV_ERR_UNKNOWN";
}

// ------------------------------------------------------------------------------ heat
adv_status adv_heat_stage(const adv_heat_desc* d, int stage, const void* u_in, const void* u_n, void* u_out,
                          void* stream) {
  ADV_NVTX_RANGE("adv_heat_stage");
  adv_status st = heat_validate(d);
  if (st != ADV_OK) return st;
  if (!u_in || !u_n || !u_out) return set_error(ADV_ERR_INVALID_ARG, "heat: null buffer");
  if (u_in == u_out) return set_error(ADV_ERR_INVALID_ARG, "heat: u_in and u_out must not alias");
  HeatLaunch L;
  st = heat_prepare(*d, u_in, &L);
  if (st != ADV_OK) return st;
  return heat_launch(*d, L, stage, u_in, u_n, u_out, static_cast<cudaStream_t>(stream));
}

adv_status adv_test_heat_stage_withheld(const adv_heat_desc* d, int stage, const void* u_in, const void* u_n,
                                        void* u_out, int plane, uint64_t wait_limit_ns, void* stream) {
  ADV_NVTX_RANGE("adv_test_heat_stage_withheld");
  adv_status st = heat_validate(d);
  if (st != ADV_OK) return st;
  if (!u_in || !u_n || !u_out) return set_error(ADV_ERR_INVALID_ARG, "heat: null buffer");
  if (u_in == u_out) return set_error(ADV_ERR_INVALID_ARG, "heat: u_in and u_out must not alias");
  const int nz = d->ndim == 3 ? d->nz : 1;
  if (plane < 0 || plane >= nz) return set_error(ADV_ERR_INVALID_ARG, "heat test: withheld plane outside the grid");
  if (wait_limit_ns < 100000ull || wait_limit_ns > kWaitLimitNs)
    return set_error(ADV_ERR_INVALID_ARG, "heat test: wait limit must lie in [1e5, 2e9] ns");
  HeatLaunch L;
  if ((st = heat_prepare(*d, u_in, &L)) != ADV_OK) return st;
  if (stage != 1 || u_n != u_in) return set_error(ADV_ERR_UNSUPPORTED, "heat test: the withheld-copy test runs stage 1");
  L.withheld_plane = plane;
  L.wait_limit_ns = wait_limit_ns;
  return heat_launch_test_hook(*d, L, u_in, u_out, static_cast<cudaStream_t>(stream));
}

adv_status adv_device_status(void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (adv_status st = reject_capture(s, "device_status"); st != ADV_OK) return st;
  return read_and_clear_device_status(s);
}

adv_status adv_heat_workspace_bytes(const adv_heat_desc* d, int time_scheme, size_t* bytes) {
  adv_status st = heat_validate(d);
  if (st != ADV_OK) return st;
  if (!bytes) return set_error(ADV_ERR_INVALID_ARG, "heat: null output");
  if (time_scheme != ADV_EULER && time_scheme != ADV_SSPRK3) return set_error(ADV_ERR_INVALID_ARG, "heat: bad time scheme");
  const size_t n = (size_t)d->nx * d->ny * (d->ndim == 3 ? d->nz : 1);
  const size_t es = d->dtype == ADV_F32 ? 4 : 8;
  const size_t one = (n * es + 255) / 256 * 256;
  *bytes = time_scheme == ADV_EULER ? one : 2 * one;
  return ADV_OK;
}

adv_status adv_heat_run(const adv_heat_desc* d, int time_scheme, int64_t nsteps, void* u, void* workspace,
                        void* stream) {
  ADV_NVTX_RANGE("adv_heat_run");
  size_t ws = 0;
  adv_status st = adv_heat_workspace_bytes(d, time_scheme, &ws);
  if (st != ADV_OK) return st;
  if (nsteps < 0) return set_error(ADV_ERR_INVALID_ARG, "heat: negative step count");
  if (!u || !workspace) return set_error(ADV_ERR_INVALID_ARG, "heat: null buffer");
  if (nsteps == 0) return ADV_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = (size_t)d->nx * d->ny * (d->ndim == 3 ? d->nz : 1);
  const size_t es = d->dtype == ADV_F32 ? 4 : 8;
  const size_t one = (n * es + 255) / 256 * 256;
  char* w1 = static_cast<char*>(workspace);
  char* w2 = w1 + one;
  const TuneParams steps = tune_lookup(TUNE_HEAT_STEPS, heat_tune_variant(*d), d->nx, d->ny, d->ndim == 3 ? d->nz : 1);
  if (time_scheme == ADV_EULER && nsteps >= 2 && steps.set && steps.a == 2 && heat2_eligible(*d, u) &&
      heat2_eligible(*d, w1)) {
    // Two steps per launch, where the autotuner measured it faster (one pass over HBM per two
    // updates): u -(2)-> w1 -(2)-> u, a chunk of 4*C steps captured once and replayed; 2 or 3
    // remaining steps end with single-step launches.
    HeatLaunch Ta, Tb, La, Lb;
    if ((st = heat2_prepare(*d, u, &Ta)) != ADV_OK) return st;
    if ((st = heat2_prepare(*d, w1, &Tb)) != ADV_OK) return st;
    if ((st = heat_prepare(*d, u, &La)) != ADV_OK) return st;
    if ((st = heat_prepare(*d, w1, &Lb)) != ADV_OK) return st;
    const int64_t quads = nsteps / 4, rem = nsteps % 4;
    const int64_t C = std::min<int64_t>(quads, 32);
    auto chunk = [&](cudaStream_t cs) -> adv_status {
      for (int64_t i = 0; i < C; ++i) {
        adv_status r = heat2_launch(*d, Ta, u, w1, cs);
        if (r != ADV_OK) return r;
        r = heat2_launch(*d, Tb, w1, u, cs);
        if (r != ADV_OK) return r;
      }
      return ADV_OK;
    };
    if (C > 0) {
      const std::string key = graph_key("heat-euler2", *d, u, workspace, C);
      if ((st = replay(key, s, quads / C, chunk, 2 * C)) != ADV_OK) return st;
      for (int64_t i = 0; i < quads % C; ++i) {
        if ((st = heat2_launch(*d, Ta, u, w1, s)) != ADV_OK) return st;
        if ((st = heat2_launch(*d, Tb, w1, u, s)) != ADV_OK) return st;
      }
    }
    if (rem == 3) {
      if ((st = heat2_launch(*d, Ta, u, w1, s)) != ADV_OK) return st;
      if ((st = heat_launch(*d, Lb, 1, w1, w1, u, s)) != ADV_OK) return st;
    } else if (rem == 2) {
      if ((st = heat_launch(*d, La, 1, u, u, w1, s)) != ADV_OK) return st;
      if ((st = heat_launch(*d, Lb, 1, w1, w1, u, s)) != ADV_OK) return st;
    } else if (rem == 1) {
      if ((st = heat_launch(*d, La, 1, u, u, w1, s)) != ADV_OK) return st;
      ADV_CUDA_TRY(cudaMemcpyAsync(u, w1, n * es, cudaMemcpyDeviceToDevice, s));
    }
  } else if (time_scheme == ADV_EULER && d->ndim == 2 && d->dtype == ADV_F32 && nsteps >= 2) {
    // 2D FP32: K steps per launch (overlapped temporal tiling in shared memory, heat2d_multi.cu;
    // 512^2 x 1000 steps: 145 vs 102 Gcell-updates/s with one step per launch),
    // ping-pong u -> w1 -> u; a chunk of 2*C launches is captured once and replayed, the
    // remaining full launch and a shorter last one run directly.
    const int K = heat2d_multi_steps();
    const int64_t full = nsteps / K;
    const int rem = (int)(nsteps % K);
    const int64_t pairs = full / 2;
    const int64_t C = std::min<int64_t>(pairs, 32);
    auto chunk = [&](cudaStream_t cs) -> adv_status {
      for (int64_t i = 0; i < C; ++i) {
        adv_status r = heat2d_multi_launch(*d, u, w1, K, cs);
        if (r != ADV_OK) return r;
        r = heat2d_multi_launch(*d, w1, u, K, cs);
        if (r != ADV_OK) return r;
      }
      return ADV_OK;
    };
    if (C > 0) {
      const std::string key = graph_key("heat2d-multi", *d, u, workspace, C);
      if ((st = replay(key, s, pairs / C, chunk, 2 * C)) != ADV_OK) return st;
      for (int64_t i = 0; i < pairs % C; ++i) {
        if ((st = heat2d_multi_launch(*d, u, w1, K, s)) != ADV_OK) return st;
        if ((st = heat2d_multi_launch(*d, w1, u, K, s)) != ADV_OK) return st;
      }
    }
    bool in_w1 = false;
    if (full % 2) {
      if ((st = heat2d_multi_launch(*d, u, w1, K, s)) != ADV_OK) return st;
      in_w1 = true;
    }
    if (rem) {
      if ((st = heat2d_multi_launch(*d, in_w1 ? w1 : u, in_w1 ? u : w1, rem, s)) != ADV_OK) return st;
      in_w1 = !in_w1;
    }
    if (in_w1) ADV_CUDA_TRY(cudaMemcpyAsync(u, w1, n * es, cudaMemcpyDeviceToDevice, s));
  } else if (time_scheme == ADV_EULER) {
    HeatLaunch La, Lb;
    if ((st = heat_prepare(*d, u, &La)) != ADV_OK) return st;
    if ((st = heat_prepare(*d, w1, &Lb)) != ADV_OK) return st;
    // Ping-pong u -> w1 -> u; a chunk of 2*C steps is captured once and replayed.
    const int64_t pairs = nsteps / 2;
    const int64_t C = std::min<int64_t>(pairs, 32);
    auto chunk = [&](cudaStream_t cs) -> adv_status {
      for (int64_t i = 0; i < C; ++i) {
        adv_status r = heat_launch(*d, La, 1, u, u, w1, cs);
        if (r != ADV_OK) return r;
        r = heat_launch(*d, Lb, 1, w1, w1, u, cs);
        if (r != ADV_OK) return r;
      }
      return ADV_OK;
    };
    if (C > 0) {
      const std::string key = graph_key("heat-euler", *d, u, workspace, C);
      if ((st = replay(key, s, pairs / C, chunk, 2 * C)) != ADV_OK) return st;
      for (int64_t i = 0; i < pairs % C; ++i) {
        if ((st = heat_launch(*d, La, 1, u, u, w1, s)) != ADV_OK) return st;
        if ((st = heat_launch(*d, Lb, 1, w1, w1, u, s)) != ADV_OK) return st;
      }
    }
    if (nsteps % 2) {
      if ((st = heat_launch(*d, La, 1, u, u, w1, s)) != ADV_OK) return st;
      ADV_CUDA_TRY(cudaMemcpyAsync(u, w1, n * es, cudaMemcpyDeviceToDevice, s));
    }
  } else {
    HeatLaunch L1, L2, L3;
    if ((st = heat_prepare(*d, u, &L1)) != ADV_OK) return st;
    if ((st = heat_prepare(*d, w1, &L2)) != ADV_OK) return st;
    if ((st = heat_prepare(*d, w2, &L3)) != ADV_OK) return st;
    auto step = [&](cudaStream_t cs) -> adv_status {
      adv_status r = heat_launch(*d, L1, 1, u, u, w1, cs);
      if (r == ADV_OK) r = heat_launch(*d, L2, 2, w1, u, w2, cs);
      if (r == ADV_OK) r = heat_launch(*d, L3, 3, w2, u, u, cs);
      return r;
    };
    const int64_t C = std::min<int64_t>(nsteps, 16);
    auto chunk = [&](cudaStream_t cs) -> adv_status {
      for (int64_t i = 0; i < C; ++i) {
        adv_status r = step(cs);
        if (r != ADV_OK) return r;
      }
      return ADV_OK;
    };
    const std::string key = graph_key("heat-rk3", *d, u, workspace, C);
    if ((st = replay(key, s, nsteps / C, chunk, 3 * C)) != ADV_OK) return st;
    for (int64_t i = 0; i < nsteps % C; ++i)
      if ((st = step(s)) != ADV_OK) return st;
  }
  ADV_CUDA_TRY(cudaGetLastError());
  return ADV_OK;
}

// --------------------------------------------------------------------------- Burgers
adv_status adv_burgers_stage(const adv_burgers_desc* d, int stage, const void* u_in, const void* u_n, void* u_out,
                             double dt, double alpha, void* maxabs_out, void* stream) {
  ADV_NVTX_RANGE("adv_burgers_stage");
  adv_status st = burgers_validate(d);
  if (st != ADV_OK) return st;
  if (!u_in || !u_n || !u_out) return set_error(ADV_ERR_INVALID_ARG, "burgers: null buffer");
  if (u_in == u_out) return set_error(ADV_ERR_INVALID_ARG, "burgers: u_in and u_out must not alias");
  BurgersLaunch L;
  if ((st = burgers_prepare(*d, u_in, &L)) != ADV_OK) return st;
  BurgersStageArgs a{};
  a.stage = stage;
  a.u_in = u_in;
  a.u_n = u_n;
  a.u_out = u_out;
  a.dt_host = dt;
  a.alpha_host = alpha;
  a.maxabs_key = maxabs_out;
  return burgers_launch(*d, L, a, static_cast<cudaStream_t>(stream));
}

static size_t burgers_state_offset(const adv_burgers_desc* d) {
  const size_t n = (size_t)d->nx * d->ny * d->nz;
  const size_t es = d->dtype == ADV_F32 ? 4 : 8;
  return 2 * ((n * es + 255) / 256 * 256);
}

adv_status adv_burgers_workspace_bytes(const adv_burgers_desc* d, size_t* bytes) {
  adv_status st = burgers_validate(d);
  if (st != ADV_OK) return st;
  if (!bytes) return set_error(ADV_ERR_INVALID_ARG, "burgers: null output");
  *bytes = burgers_state_offset(d) + (sizeof(BurgersLoopState) + 255) / 256 * 256;
  return ADV_OK;
}

adv_status adv_burgers_run(const adv_burgers_desc* d, void* u, void* workspace, double tEnd, double cfl, int dt_rule,
                           double C, int64_t max_steps, double* t_out, int64_t* steps_out, void* stream) {
  return adv_burgers_resume(d, u, workspace, 0.0, 0, tEnd, cfl, dt_rule, C, max_steps, t_out, steps_out, stream);
}

adv_status adv_burgers_resume(const adv_burgers_desc* d, void* u, void* workspace, double t0, int64_t step0,
                              double tEnd, double cfl, int dt_rule, double C, int64_t max_steps, double* t_out,
                              int64_t* steps_out, void* stream) {
  ADV_NVTX_RANGE("adv_burgers_resume");
  adv_status st = burgers_validate(d);
  if (st != ADV_OK) return st;
  if (!u || !workspace) return set_error(ADV_ERR_INVALID_ARG, "burgers: null buffer");
  if (dt_rule != ADV_DT_FIXED && dt_rule != ADV_DT_MAXU) return set_error(ADV_ERR_INVALID_ARG, "burgers: bad dt rule");
  if (!(cfl > 0) || !std::isfinite(tEnd) || max_steps < 0) return set_error(ADV_ERR_INVALID_ARG, "burgers: bad cfl/tEnd/max_steps");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if ((st = reject_capture(s, "burgers run")) != ADV_OK) return st;
  const size_t es = d->dtype == ADV_F32 ? 4 : 8;
  const size_t n = (size_t)d->nx * d->ny * d->nz;
  const size_t one = (n * es + 255) / 256 * 256;
  char* w1 = static_cast<char*>(workspace);
  char* w2 = w1 + one;
  BurgersLoopState* dst = reinterpret_cast<BurgersLoopState*>(w1 + burgers_state_offset(d));

  if (!std::isfinite(t0) || step0 < 0) return set_error(ADV_ERR_INVALID_ARG, "burgers: bad t0/step0");
  BurgersLoopState h = burgers_loop_state(*d, tEnd, cfl, dt_rule, C, max_steps);
  h.t = t0;  // a resumed run continues the same time sum and step count
  h.step = step0;
  ADV_CUDA_TRY(cudaMemcpyAsync(dst, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  ADV_CUDA_TRY(cudaStreamSynchronize(s));
  void* key0 = d->dtype == ADV_F32 ? (void*)&dst->maxbits[0] : (void*)&dst->maxbits64[0];
  void* key1 = d->dtype == ADV_F32 ? (void*)&dst->maxbits[1] : (void*)&dst->maxbits64[1];
  void* key2 = d->dtype == ADV_F32 ? (void*)&dst->maxbits[2] : (void*)&dst->maxbits64[2];
  if ((st = max_abs_launch(d->dtype, u, (int64_t)n, key0, s)) != ADV_OK) return st;

  BurgersLaunch L1, L2, L3;
  if ((st = burgers_prepare(*d, u, &L1)) != ADV_OK) return st;
  if ((st = burgers_prepare(*d, w1, &L2)) != ADV_OK) return st;
  if ((st = burgers_prepare(*d, w2, &L3)) != ADV_OK) return st;

  auto body = [&](cudaStream_t cs, unsigned long long cond, int use_cond) -> adv_status {
    adv_status r = burgers_loop_begin_step(dst, d->dtype, cond, use_cond, cs);
    if (r != ADV_OK) return r;
    BurgersStageArgs a{};
    a.dt_dev = &dst->dt;
    a.active = &dst->active;
    a.stage = 1; a.u_in = u; a.u_n = u; a.u_out = w1; a.alpha_dev = &dst->alpha0; a.maxabs_key = key1;
    if ((r = burgers_launch(*d, L1, a, cs)) != ADV_OK) return r;
    a.stage = 2; a.u_in = w1; a.u_n = u; a.u_out = w2; a.alpha_dev = nullptr; a.alpha_key = key1; a.maxabs_key = key2;
    if ((r = burgers_launch(*d, L2, a, cs)) != ADV_OK) return r;
    a.stage = 3; a.u_in = w2; a.u_n = u; a.u_out = u; a.alpha_key = key2; a.maxabs_key = key0;
    return burgers_launch(*d, L3, a, cs);
  };

  const bool can_loop = max_steps > 0 && tEnd > 0.0;
  if (can_loop) {
    // One graph: a while-conditional node whose body is one step; the condition is set on the
    // device by the step-start kernel. Cached per (device, descriptor, buffers).
    const std::string wkey = graph_key("burgers-while", *d, u, workspace);
    cudaGraphExec_t ge = g_graphs.get(wkey);
    cudaError_t e = cudaSuccess;
    if (!ge) {
      cudaStream_t cs;
      ADV_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t g = nullptr;
      e = cudaGraphCreate(&g, 0);
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
          const int64_t before = g_launches.load();
          bst = body(cs, (unsigned long long)h_cond, 1);
          g_launches.store(before);
          cudaGraph_t outg = nullptr;
          e = cudaStreamEndCapture(cs, &outg);
        }
        if (e == cudaSuccess && bst == ADV_OK) e = cudaGraphInstantiate(&ge, g, 0);
      }
      if (g) cudaGraphDestroy(g);
      cudaStreamDestroy(cs);
      if (bst != ADV_OK) return bst;
      if (e == cudaSuccess && ge) g_graphs.put(wkey, ge);
      else ge = nullptr;
    }
    if (ge) {
      e = cudaGraphLaunch(ge, s);
      if (e != cudaSuccess) return cuda_error(e, "burgers: graph launch");
    } else {
      cudaGetLastError();  // conditional nodes unavailable: clear the non-sticky error
      // Fallback: fixed chunks of predicated steps, replayed until the device clears `active`.
      const int64_t Cch = std::min<int64_t>(max_steps, 8);
      auto chunk = [&](cudaStream_t c2) -> adv_status {
        for (int64_t i = 0; i < Cch; ++i) {
          adv_status r = body(c2, 0, 0);
          if (r != ADV_OK) return r;
        }
        return ADV_OK;
      };
      const std::string key = graph_key("burgers-chunk", *d, u, workspace, Cch);
      int64_t done = 0;
      while (done < max_steps) {
        if ((st = replay(key, s, 1, chunk, 4 * Cch)) != ADV_OK) return st;
        done += Cch;
        int active = 0;
        ADV_CUDA_TRY(cudaMemcpyAsync(&active, &dst->active, sizeof(int), cudaMemcpyDeviceToHost, s));
        ADV_CUDA_TRY(cudaStreamSynchronize(s));
        if (!active) break;
      }
    }
  }
  ADV_CUDA_TRY(cudaMemcpyAsync(&h, dst, sizeof(h), cudaMemcpyDeviceToHost, s));
  ADV_CUDA_TRY(cudaStreamSynchronize(s));
  count_launches(4 * (h.step - step0));
  if (t_out) *t_out = h.t;
  if (steps_out) *steps_out = h.step;
  return read_and_clear_device_status(s);
}

// ------------------------------------------------------------------------ reduction
adv_status adv_max_abs(int dtype, const void* u, int64_t n, double* out, void* stream) {
  ADV_NVTX_RANGE("adv_max_abs");
  if (dtype != ADV_F32 && dtype != ADV_F64) return set_error(ADV_ERR_INVALID_ARG, "max_abs: bad dtype");
  if (!u || !out || n < 0) return set_error(ADV_ERR_INVALID_ARG, "max_abs: bad arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (adv_status st = reject_capture(s, "max_abs"); st != ADV_OK) return st;
  if (n == 0) { *out = 0.0; return ADV_OK; }
  unsigned long long* acc = nullptr;
  ADV_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&acc), sizeof(unsigned long long), s));
  adv_status st = ADV_OK;
  cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) st = cuda_error(e, "max_abs: memset");
  if (st == ADV_OK) st = max_abs_launch(dtype, u, n, acc, s);
  unsigned long long key = 0;
  if (st == ADV_OK) {
    e = cudaMemcpyAsync(&key, acc, sizeof(key), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_error(e, "max_abs: read back");
  }
  cudaFreeAsync(acc, s);
  if (st != ADV_OK) return st;
  if ((st = read_and_clear_device_status(s)) != ADV_OK) return st;
  if (dtype == ADV_F32) {
    unsigned k32 = (unsigned)key;
    float f;
    std::memcpy(&f, &k32, 4);
    *out = f;
  } else {
    double v;
    std::memcpy(&v, &key, 8);
    *out = v;
  }
  return ADV_OK;
}

// ----------------------------------------------------------------- initial conditions
// Philox4x32-10 (Salmon et al., SC'11), counter-based. Draw i of stream s with seed k gives two
// uniforms in [0,1) with 53-bit resolution from the four output words.
static void philox(const uint32_t in[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  for (int r = 0; r < 10; ++r) {
    const uint64_t a = (uint64_t)0xD2511F53u * c0, b = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(b >> 32) ^ c1 ^ k0, n2 = (uint32_t)(a >> 32) ^ c3 ^ k1;
    c1 = (uint32_t)b;
    c3 = (uint32_t)a;
    c0 = n0;
    c2 = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
static void uniform2(uint32_t seed, uint32_t stream, uint64_t i, double* a, double* b) {
  const uint32_t ctr[4] = {(uint32_t)i, (uint32_t)(i >> 32), 0u, 0u};
  uint32_t o[4];
  philox(ctr, seed, stream, o);
  const double s = 1.0 / 9007199254740992.0;
  *a = (double)(((uint64_t)o[0] << 21) ^ (uint64_t)(o[1] >> 11)) * s;
  *b = (double)(((uint64_t)o[2] << 21) ^ (uint64_t)(o[3] >> 11)) * s;
}

adv_status adv_ic_heat_ref(int ndim, int nx, int ny, int nz, double dx, double dy, double dz, double* u) {
  if ((ndim != 2 && ndim != 3) || nx < 1 || ny < 1 || (ndim == 3 && nz < 1) || !u)
    return set_error(ADV_ERR_INVALID_ARG, "ic_heat_ref: bad arguments");
  const int NZ = ndim == 3 ? nz : 1;
  for (int k = 0; k < NZ; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double r2 = (-5 + i * dx) * (-5 + i * dx) + (-5 + j * dy) * (-5 + j * dy);
        if (ndim == 3) r2 += (-5 + k * dz) * (-5 + k * dz);
        bool face = i == 0 || i == nx - 1 || j == 0 || j == ny - 1;
        if (ndim == 3) face = face || k == 0 || k == nz - 1;
        u[(size_t)i + (size_t)nx * j + (size_t)nx * ny * k] = face ? 0.0 : std::exp(-(r2) / (4 * 1.0 * 0.1));
      }
  return ADV_OK;
}

adv_status adv_ic_heat2d_gauss_noise(int nx, int ny, uint32_t seed, double sigma, double* u) {
  if (nx < 2 || ny < 2 || !u) return set_error(ADV_ERR_INVALID_ARG, "ic_heat2d: bad arguments");
  const double hx = 1.0 / (nx - 1), hy = 1.0 / (ny - 1);
  const double two_pi = 6.283185307179586476925286766559;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const size_t o = (size_t)i + (size_t)nx * j;
      const double x = i * hx, y = j * hy;
      double a, b;
      uniform2(seed, 1u, (uint64_t)o, &a, &b);
      const double g = std::exp(-((x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5)) / 0.01);
      const double z = std::sqrt(-2.0 * std::log(1.0 - a)) * std::cos(two_pi * b);
      const bool edge = i == 0 || i == nx - 1 || j == 0 || j == ny - 1;
      u[o] = edge ? 0.0 : g + sigma * z;
    }
  return ADV_OK;
}

adv_status adv_ic_heat3d_blobs(int nx, int ny, int nz, uint32_t seed, int nblobs, double* u) {
  if (nx < 2 || ny < 2 || nz < 2 || nblobs < 0 || !u) return set_error(ADV_ERR_INVALID_ARG, "ic_heat3d: bad arguments");
  std::vector<double> c(4 * (size_t)nblobs);
  for (int m = 0; m < nblobs; ++m) {
    double a, b, e, f;
    uniform2(seed, 2u, (uint64_t)(2 * m), &a, &b);
    uniform2(seed, 2u, (uint64_t)(2 * m + 1), &e, &f);
    c[4 * m] = 0.2 + 0.6 * a;
    c[4 * m + 1] = 0.2 + 0.6 * b;
    c[4 * m + 2] = 0.2 + 0.6 * e;
    c[4 * m + 3] = 0.02 + 0.06 * f;
  }
  const double hx = 1.0 / (nx - 1), hy = 1.0 / (ny - 1), hz = 1.0 / (nz - 1);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const bool face = i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k == nz - 1;
        double s = 0.0;
        if (!face) {
          const double x = i * hx, y = j * hy, z = k * hz;
          for (int m = 0; m < nblobs; ++m) {
            const double ddx = x - c[4 * m], ddy = y - c[4 * m + 1], ddz = z - c[4 * m + 2], sg = c[4 * m + 3];
            s += std::exp(-(ddx * ddx + ddy * ddy + ddz * ddz) / (2 * sg * sg));
          }
        }
        u[(size_t)i + (size_t)nx * j + (size_t)nx * ny * k] = s;
      }
  return ADV_OK;
}

adv_status adv_ic_burgers_fourier(int nx, int ny, int nz, double L, uint32_t seed, int nmodes, double amax, double* u) {
  if (nx < 1 || ny < 1 || nz < 1 || nmodes < 0 || !(L > 0) || !u)
    return set_error(ADV_ERR_INVALID_ARG, "ic_burgers_fourier: bad arguments");
  const double two_pi = 6.283185307179586476925286766559;
  const double pi = 3.14159265358979323846264338327950288;
  std::vector<double> md(5 * (size_t)nmodes);
  uint64_t idx = 0;
  for (int m = 0; m < nmodes; ++m) {
    int n1, n2, n3;
    for (;;) {  // wave vector uniform over {n in [-4,4]^3 : 0 < |n| <= 4} by rejection
      double a, b, c, e;
      uniform2(seed, 3u, idx++, &a, &b);
      uniform2(seed, 3u, idx++, &c, &e);
      n1 = (int)std::floor(a * 9.0) - 4;
      n2 = (int)std::floor(b * 9.0) - 4;
      n3 = (int)std::floor(c * 9.0) - 4;
      const int r2 = n1 * n1 + n2 * n2 + n3 * n3;
      if (r2 > 0 && r2 <= 16) break;
    }
    double a, b;
    uniform2(seed, 4u, (uint64_t)m, &a, &b);
    md[5 * m] = n1; md[5 * m + 1] = n2; md[5 * m + 2] = n3;
    md[5 * m + 3] = amax * a;
    md[5 * m + 4] = two_pi * b;
  }
  const double hx = L / nx, hy = L / ny, hz = L / nz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double x = (i + 0.5) * hx, y = (j + 0.5) * hy, z = (k + 0.5) * hz;
        double s = 0.5;
        for (int m = 0; m < nmodes; ++m)
          s += md[5 * m + 3] * std::cos(pi * (md[5 * m] * x + md[5 * m + 1] * y + md[5 * m + 2] * z) + md[5 * m + 4]);
        u[(size_t)i + (size_t)nx * j + (size_t)nx * ny * k] = s;
      }
  return ADV_OK;
}

adv_status adv_ic_burgers_ref(int nx, int ny, int nz, double dx, double dy, double dz, double* u) {
  if (nx < 1 || ny < 1 || nz < 1 || !u) return set_error(ADV_ERR_INVALID_ARG, "ic_burgers_ref: bad arguments");
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double x = i * dx, y = j * dy, z = k * dz;
        u[(size_t)i + (size_t)nx * j + (size_t)nx * ny * k] =
            1.0 * std::exp(-((x - 1.0) * (x - 1.0) + (y - 1.0) * (y - 1.0) + (z - 1.0) * (z - 1.0)) / 0.1);
      }
  return ADV_OK;
}

adv_status adv_ic_burgers_ref2d(int nx, int ny, double dx, double dy, double* u) {
  if (nx < 1 || ny < 1 || !u) return set_error(ADV_ERR_INVALID_ARG, "ic_burgers_ref2d: bad arguments");
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const double x = (0.5 * (nx - 1) - i) * dx, y = (0.5 * (ny - 1) - j) * dy;
      const bool ring = i == 0 || i == nx - 1 || j == 0 || j == ny - 1;
      u[(size_t)i + (size_t)nx * j] = ring ? 0.0 : 1.0 * std::exp(-((x * x) + (y * y)) / 0.1);
    }
  return ADV_OK;
}

adv_status adv_write_result_bin(const char* path, int dtype, const void* host_u, int64_t n) {
  if (!path || !host_u || n < 0 || (dtype != ADV_F32 && dtype != ADV_F64))
    return set_error(ADV_ERR_INVALID_ARG, "write_result_bin: bad arguments");
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(ADV_ERR_INVALID_ARG, std::string("write_result_bin: cannot open ") + path);
  std::vector<float> buf(1 << 16);
  int64_t done = 0;
  while (done < n) {
    const int64_t m = std::min<int64_t>(n - done, (int64_t)buf.size());
    for (int64_t i = 0; i < m; ++i)
      buf[i] = dtype == ADV_F32 ? static_cast<const float*>(host_u)[done + i]
                                : (float)static_cast<const double*>(host_u)[done + i];
    if (std::fwrite(buf.data(), sizeof(float), (size_t)m, f) != (size_t)m) {
      std::fclose(f);
      return set_error(ADV_ERR_INVALID_ARG, "write_result_bin: short write");
    }
    done += m;
  }
  std::fclose(f);
  return ADV_OK;
}

}  // extern "C"
