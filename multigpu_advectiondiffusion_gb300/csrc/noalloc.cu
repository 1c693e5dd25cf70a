// noalloc.cu -- adv_heat_run_noalloc (include/advdiff.h): the heat time loop for callers that
// cannot allocate device memory. Its intermediate state lives in the file-scope array below
// instead of a caller- or library-allocated workspace; the stages are launched one by one on the
// caller's stream with no graph, no stream and no allocation.
#include <mutex>
#include <string>

#include "adv_internal.h"
#include "nvtx_range.h"

namespace adv {

// Scratch of adv_heat_run_noalloc. Every GPU that loads this library holds it until exit.
static __device__ __align__(256) unsigned char g_noalloc_scratch[ADV_NOALLOC_SCRATCH_BYTES];

// Unique id of the calling thread's current CUDA context (0 if none is current), through the
// driver entry points the runtime exposes (no -lcuda link).
static unsigned long long current_context_id() {
  typedef CUresult (*GetCurrentFn)(CUcontext*);
  typedef CUresult (*GetIdFn)(CUcontext, unsigned long long*);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrentFn>(p);
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetIdFn>(p);
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of g_noalloc_scratch on the current device. In host code the symbol itself is
// only a host-side stand-in, so its address is looked up (with that device current) once per
// device and context, and cached next to the context's unique id: after a cudaDeviceReset the
// device has a new context, in which the array has a new address, and the lookup is made again.
static adv_status noalloc_scratch(void** out) {
  static std::mutex mu;
  static void* addr[64] = {};
  static unsigned long long ctx_of[64] = {};
  int dev = -1;
  ADV_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(ADV_ERR_UNSUPPORTED, "heat_run_noalloc: device ordinal out of range");
  std::lock_guard<std::mutex> lk(mu);
  const unsigned long long ctx = current_context_id();
  if (!addr[dev] || ctx == 0 || ctx != ctx_of[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "heat_run_noalloc: cudaGetSymbolAddress of the scratch array");
    addr[dev] = p;
    ctx_of[dev] = current_context_id();  // the lookup made the device's context current
  }
  *out = addr[dev];
  return ADV_OK;
}

}  // namespace adv

using namespace adv;

extern "C" adv_status adv_heat_run_noalloc(const adv_heat_desc* d, int time_scheme, int64_t nsteps, void* u,
                                           void* stream) {
  ADV_NVTX_RANGE("adv_heat_run_noalloc");
  size_t need = 0;
  adv_status st = adv_heat_workspace_bytes(d, time_scheme, &need);
  if (st != ADV_OK) return st;
  if (need > ADV_NOALLOC_SCRATCH_BYTES)
    return set_error(ADV_ERR_INVALID_ARG, "heat_run_noalloc: this run needs " + std::to_string(need) +
                                              " bytes of scratch; the fixed scratch array holds " +
                                              std::to_string((size_t)ADV_NOALLOC_SCRATCH_BYTES) + " bytes");
  if (nsteps < 0) return set_error(ADV_ERR_INVALID_ARG, "heat_run_noalloc: negative step count");
  if (!u) return set_error(ADV_ERR_INVALID_ARG, "heat_run_noalloc: null buffer");
  if (nsteps == 0) return ADV_OK;
  void* ws = nullptr;
  if ((st = noalloc_scratch(&ws)) != ADV_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = (size_t)d->nx * d->ny * (d->ndim == 3 ? d->nz : 1);
  const size_t es = d->dtype == ADV_F32 ? 4 : 8;
  const size_t one = (n * es + 255) / 256 * 256;
  char* w1 = static_cast<char*>(ws);
  char* w2 = w1 + one;
  if (time_scheme == ADV_EULER) {
    HeatLaunch La, Lb;
    if ((st = heat_prepare(*d, u, &La)) != ADV_OK) return st;
    if ((st = heat_prepare(*d, w1, &Lb)) != ADV_OK) return st;
    for (int64_t i = 0; i < nsteps / 2; ++i) {
      if ((st = heat_launch(*d, La, 1, u, u, w1, s)) != ADV_OK) return st;
      if ((st = heat_launch(*d, Lb, 1, w1, w1, u, s)) != ADV_OK) return st;
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
    for (int64_t i = 0; i < nsteps; ++i) {
      if ((st = heat_launch(*d, L1, 1, u, u, w1, s)) != ADV_OK) return st;
      if ((st = heat_launch(*d, L2, 2, w1, u, w2, s)) != ADV_OK) return st;
      if ((st = heat_launch(*d, L3, 3, w2, u, u, s)) != ADV_OK) return st;
    }
  }
  ADV_CUDA_TRY(cudaGetLastError());
  return ADV_OK;
}
