// autotune.cu -- the launch-shape autotuner (adv_autotune_* in advdiff.h) and its table.
//
// The stage kernels' tiles are fixed by the hardware geometry they are built around (a warp of
// 16-byte vectors in x, register windows in z), but how the work is cut is not: the heat and
// Burgers stages run one wave of CTAs over equal shares of (tile, z-plane) pairs, and the share
// size trades z-halo re-reads (short shares) against tail imbalance and latency hiding (few
// CTAs); the heat-with-k(x) kernels march a z chunk per CTA with a tunable block height. For a
// given problem the tuner times every candidate on the caller's data (out of place, into a
// temporary buffer, so the state is untouched), keeps the fastest, and the launchers use it from
// then on (per device and problem shape, for the life of the process). Cached CUDA graphs are
// dropped when a choice changes because they hold the old launch shapes.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "adv_internal.h"
#include "nvtx_range.h"

namespace adv {

adv_status heatk_validate_desc(const adv_heatk_desc* d);
adv_status heatk_step_run(const adv_heatk_desc& d, const void* k, const void* u_in, void* u_out, cudaStream_t s);
adv_status heatk_adjoint_run(const adv_heatk_desc& d, const void* k, const void* u_n, const void* lam_next,
                             void* lam_out, void* grad_k, cudaStream_t s);

namespace {

using Key = std::tuple<int, int, int, int, int, int>;  // device, kind, variant, nx, ny, nz
std::mutex g_mu;
std::map<Key, TuneParams> g_table;

int current_device() {
  int d = -1;
  cudaGetDevice(&d);
  return d;
}

// Mean time of `reps` calls of fn on stream s (after one warm-up call), in microseconds.
template <class F>
adv_status time_us(F fn, int reps, cudaStream_t s, double* us) {
  adv_status st = fn();
  if (st != ADV_OK) return st;
  cudaEvent_t a, b;
  ADV_CUDA_TRY(cudaEventCreate(&a));
  cudaError_t e = cudaEventCreate(&b);
  if (e != cudaSuccess) {
    cudaEventDestroy(a);
    return cuda_error(e, "autotune: event");
  }
  e = cudaEventRecord(a, s);
  for (int i = 0; e == cudaSuccess && st == ADV_OK && i < reps; ++i) st = fn();
  if (e == cudaSuccess) e = cudaEventRecord(b, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (st != ADV_OK) return st;
  if (e != cudaSuccess) return cuda_error(e, "autotune: timing");
  *us = 1e3 * ms / reps;
  return ADV_OK;
}

struct Candidate {
  int a, b;
};

// Times every candidate (stored in the table while it runs) and keeps the fastest. prep()
// resolves the launch for the candidate once (host work: tensor maps, attributes); run() only
// launches, so the timing is the kernel's and not the host's.
template <class P, class F>
adv_status sweep(int kind, int variant, int nx, int ny, int nz, const std::vector<Candidate>& cands, Candidate dflt,
                 P prep, F run, int reps, cudaStream_t s, adv_tune_result* out) {
  const int dev = current_device();
  const Key key{dev, kind, variant, nx, ny, nz};
  TuneParams saved;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_table.find(key);
    if (it != g_table.end()) saved = it->second;
  }
  double best = 1e300, at_default = 0.0;
  Candidate pick = dflt;
  Candidate fastest = dflt;
  adv_status st = ADV_OK;
  for (const Candidate& c : cands) {
    tune_store(kind, variant, nx, ny, nz, TuneParams{c.a, c.b, true});
    double us = 0.0;
    st = prep();
    if (st == ADV_OK) st = time_us(run, reps, s, &us);
    if (st != ADV_OK) break;
    if (c.a == dflt.a && c.b == dflt.b) at_default = us;
    if (us < best) {
      best = us;
      fastest = c;
    }
  }
  // keep the default unless a candidate beats it clearly (run-to-run noise is ~1%)
  pick = (at_default > 0.0 && best > 0.98 * at_default) ? dflt : fastest;
  if (pick.a == dflt.a && pick.b == dflt.b && at_default > 0.0) best = at_default;
  if (st != ADV_OK) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (saved.set) g_table[key] = saved;
    else g_table.erase(key);
    return st;
  }
  tune_store(kind, variant, nx, ny, nz, TuneParams{pick.a, pick.b, true});
  graph_cache_clear();
  if (out) {
    out->kind = kind;
    out->param_a = pick.a;
    out->param_b = pick.b;
    out->candidates = (int32_t)cands.size();
    out->best_us = best;
    out->default_us = at_default;
  }
  return ADV_OK;
}

// A temporary device buffer released on scope exit (stream ordered).
struct Scratch {
  void* p = nullptr;
  cudaStream_t s;
  explicit Scratch(cudaStream_t st) : s(st) {}
  adv_status alloc(size_t bytes) {
    ADV_CUDA_TRY(cudaMallocAsync(&p, bytes, s));
    return ADV_OK;
  }
  ~Scratch() {
    if (p) cudaFreeAsync(p, s);
  }
};

}  // namespace

TuneParams tune_lookup(int kind, int variant, int nx, int ny, int nz) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_table.find(Key{current_device(), kind, variant, nx, ny, nz});
  return it == g_table.end() ? TuneParams{} : it->second;
}

void tune_store(int kind, int variant, int nx, int ny, int nz, TuneParams p) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_table[Key{current_device(), kind, variant, nx, ny, nz}] = p;
}

void tune_clear() {
  std::lock_guard<std::mutex> lk(g_mu);
  g_table.clear();
}

}  // namespace adv

using namespace adv;

extern "C" {

adv_status adv_autotune_heat(const adv_heat_desc* d, const void* u, void* stream, adv_tune_result* out) {
  ADV_NVTX_RANGE("adv_autotune_heat");
  adv_status st = heat_validate(d);
  if (st != ADV_OK) return st;
  if (!u) return set_error(ADV_ERR_INVALID_ARG, "autotune: null buffer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nz = d->ndim == 3 ? d->nz : 1;
  const size_t bytes = (size_t)d->nx * d->ny * nz * (d->dtype == ADV_F32 ? 4 : 8);
  // Time stages the way a run issues them: each launch reads the previous launch's output
  // (two scratch arrays, the first a copy of u; u itself is not modified).
  Scratch tmp(s), tmp2(s);
  if ((st = tmp.alloc(bytes)) != ADV_OK) return st;
  if ((st = tmp2.alloc(bytes)) != ADV_OK) return st;
  ADV_CUDA_TRY(cudaMemcpyAsync(tmp2.p, u, bytes, cudaMemcpyDeviceToDevice, s));
  // occupancy of the stage kernel bounds the CTAs per SM
  HeatLaunch L;
  if ((st = heat_prepare(*d, u, &L)) != ADV_OK) return st;
  const int occ = std::max(1, L.occ);
  std::vector<Candidate> cands;
  const int shares2[] = {1, 2, 4, 8};
  const int shares3[] = {4, 8, 16, 32};
  for (int a = 1; a <= std::max(occ, 1); ++a)
    for (int b : (d->ndim == 3 ? shares3 : shares2)) cands.push_back({a, b});
  const Candidate dflt{occ, d->ndim == 3 ? 8 : 1};
  const size_t cells = (size_t)d->nx * d->ny * nz;
  const int reps = (int)std::max<size_t>(10, std::min<size_t>(200, ((size_t)256 << 20) / std::max<size_t>(cells, 1)));
  HeatLaunch La, Lb;
  int flip = 0;
  auto prep = [&]() {
    adv_status r = heat_prepare(*d, tmp2.p, &La);
    return r == ADV_OK ? heat_prepare(*d, tmp.p, &Lb) : r;
  };
  auto run = [&]() {
    flip ^= 1;
    return flip ? heat_launch(*d, La, 1, tmp2.p, tmp2.p, tmp.p, s) : heat_launch(*d, Lb, 1, tmp.p, tmp.p, tmp2.p, s);
  };
  return sweep(TUNE_HEAT, heat_tune_variant(*d), d->nx, d->ny, nz, cands, dflt, prep, run, reps, s, out);
}

adv_status adv_autotune_burgers(const adv_burgers_desc* d, const void* u, void* stream, adv_tune_result* out) {
  ADV_NVTX_RANGE("adv_autotune_burgers");
  adv_status st = burgers_validate(d);
  if (st != ADV_OK) return st;
  if (!u) return set_error(ADV_ERR_INVALID_ARG, "autotune: null buffer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t cells = (size_t)d->nx * d->ny * d->nz;
  Scratch tmp(s);
  if ((st = tmp.alloc(cells * (d->dtype == ADV_F32 ? 4 : 8))) != ADV_OK) return st;
  BurgersLaunch L;
  if ((st = burgers_prepare(*d, u, &L)) != ADV_OK) return st;
  const int occ = std::max(1, L.occ);
  std::vector<Candidate> cands;
  for (int a = 1; a <= occ; ++a)
    for (int b : {4, 8, 16, 32}) cands.push_back({a, b});
  const Candidate dflt{occ, 8};
  const int reps = (int)std::max<size_t>(3, std::min<size_t>(20, ((size_t)32 << 20) / std::max<size_t>(cells, 1)));
  BurgersLaunch Lc;
  BurgersStageArgs a{};
  a.stage = 1;
  a.u_in = u;
  a.u_n = u;
  a.u_out = tmp.p;
  a.dt_host = 1e-6;
  a.alpha_host = 1.0;
  auto prep = [&]() { return burgers_prepare(*d, u, &Lc); };
  auto run = [&]() { return burgers_launch(*d, Lc, a, s); };
  return sweep(TUNE_BURGERS, burgers_tune_variant(*d), d->nx, d->ny, d->nz, cands, dflt, prep, run, reps, s, out);
}

adv_status adv_autotune_heatk(const adv_heatk_desc* d, const void* k, const void* u, void* stream,
                              adv_tune_result* out_step, adv_tune_result* out_adjoint) {
  ADV_NVTX_RANGE("adv_autotune_heatk");
  adv_status st = heatk_validate_desc(d);
  if (st != ADV_OK) return st;
  if (!k || !u) return set_error(ADV_ERR_INVALID_ARG, "autotune: null buffer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t cells = (size_t)d->nx * d->ny * d->nz;
  const size_t bytes = cells * (d->dtype == ADV_F32 ? 4 : 8);
  Scratch tmp(s), grad(s);
  if ((st = tmp.alloc(bytes)) != ADV_OK) return st;
  if ((st = grad.alloc(bytes)) != ADV_OK) return st;
  ADV_CUDA_TRY(cudaMemsetAsync(grad.p, 0, bytes, s));
  std::vector<Candidate> cands;
  for (int a : {4, 8, 16})
    for (int b : {4, 8, 16, 32}) cands.push_back({a, b});
  const Candidate dflt{8, 16};
  const int reps = (int)std::max<size_t>(3, std::min<size_t>(50, ((size_t)64 << 20) / std::max<size_t>(cells, 1)));
  auto none = []() { return ADV_OK; };  // the heat-k launch shape is resolved per call (no host setup)
  auto step = [&]() { return heatk_step_run(*d, k, u, tmp.p, s); };
  st = sweep(TUNE_HEATK_STEP, d->dtype, d->nx, d->ny, d->nz, cands, dflt, none, step, reps, s, out_step);
  if (st != ADV_OK) return st;
  // the adjoint reads u as both the state and the incoming adjoint (values do not matter here)
  auto adj = [&]() { return heatk_adjoint_run(*d, k, u, u, tmp.p, grad.p, s); };
  return sweep(TUNE_HEATK_ADJ, d->dtype, d->nx, d->ny, d->nz, cands, dflt, none, adj, reps, s, out_adjoint);
}

adv_status adv_autotune_clear(void) {
  tune_clear();
  graph_cache_clear();
  return ADV_OK;
}

}  // extern "C"
