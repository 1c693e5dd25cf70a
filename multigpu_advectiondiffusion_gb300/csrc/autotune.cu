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
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <map>
#include <mutex>
#include <string>
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

// ------------------------------------------------------------------ table export / import
// The table of this device as JSON, so a tuned set of shapes can be kept between processes:
//   {"advdiff_autotune": 1, "entries": [{"kind": 1, "variant": 5, "nx": 256, "ny": 256,
//    "nz": 256, "a": 4, "b": 8}, ...]}
// An import accepts only values the tuner itself tries (the launch shapes the kernels are
// tested with), so a stale or edited file cannot produce an untested launch.
namespace {

bool tune_allowed(int kind, long long a, long long b) {
  auto in = [](long long v, std::initializer_list<int> set) {
    return std::find(set.begin(), set.end(), (int)v) != set.end() && v == (int)v;
  };
  switch (kind) {
    case TUNE_HEAT: return a >= 1 && a <= 32 && in(b, {1, 2, 4, 8, 16, 32});
    case TUNE_BURGERS: return a >= 1 && a <= 32 && in(b, {4, 8, 16, 32});
    case TUNE_HEATK_STEP:
    case TUNE_HEATK_ADJ: return in(a, {4, 8, 16}) && in(b, {4, 8, 16, 32});
    case TUNE_HEAT_STEPS: return in(a, {1, 2}) && b == 1;
    default: return false;
  }
}

// Reader for the export format only: objects with identifier keys, integer values and the one
// array of entry objects. Anything else fails.
struct TuneJson {
  const char* p;
  void ws() {
    while (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r') ++p;
  }
  bool lit(char c) {
    ws();
    if (*p != c) return false;
    ++p;
    return true;
  }
  bool key(std::string* out) {
    if (!lit('"')) return false;
    const char* b = p;
    while (*p && (std::isalnum((unsigned char)*p) || *p == '_')) ++p;
    if (*p != '"' || p == b) return false;
    out->assign(b, (size_t)(p - b));
    ++p;
    return lit(':');
  }
  bool integer(long long* v) {
    ws();
    if (!(*p == '-' || std::isdigit((unsigned char)*p))) return false;
    char* end = nullptr;
    errno = 0;
    const long long x = std::strtoll(p, &end, 10);
    if (end == p || errno) return false;
    p = end;
    *v = x;
    return true;
  }
};

struct TuneEntry {
  int kind, variant, nx, ny, nz;
  TuneParams p;
};

bool parse_entry(TuneJson& j, TuneEntry* e) {
  if (!j.lit('{')) return false;
  const char* names[7] = {"kind", "variant", "nx", "ny", "nz", "a", "b"};
  long long v[7];
  bool seen[7] = {false, false, false, false, false, false, false};
  do {
    std::string k;
    long long x;
    if (!j.key(&k) || !j.integer(&x)) return false;
    int i = 0;
    while (i < 7 && k != names[i]) ++i;
    if (i == 7 || seen[i]) return false;
    seen[i] = true;
    v[i] = x;
  } while (j.lit(','));
  if (!j.lit('}')) return false;
  for (bool b : seen)
    if (!b) return false;
  for (int i = 1; i < 5; ++i)
    if (v[i] < 0 || v[i] > (1 << 24)) return false;
  if (v[2] < 1 || v[3] < 1 || v[4] < 1 || !tune_allowed((int)v[0], v[5], v[6])) return false;
  *e = TuneEntry{(int)v[0], (int)v[1], (int)v[2], (int)v[3], (int)v[4], TuneParams{(int)v[5], (int)v[6], true}};
  return true;
}

bool parse_table(const char* text, std::vector<TuneEntry>* out) {
  TuneJson j{text};
  if (!j.lit('{')) return false;
  bool version = false, entries = false;
  do {
    std::string k;
    if (!j.key(&k)) return false;
    if (k == "advdiff_autotune" && !version) {
      long long x;
      if (!j.integer(&x) || x != 1) return false;
      version = true;
    } else if (k == "entries" && !entries) {
      if (!j.lit('[')) return false;
      if (!j.lit(']')) {
        do {
          TuneEntry e;
          if (!parse_entry(j, &e)) return false;
          out->push_back(e);
        } while (j.lit(','));
        if (!j.lit(']')) return false;
      }
      entries = true;
    } else {
      return false;
    }
  } while (j.lit(','));
  if (!j.lit('}') || !version || !entries) return false;
  j.ws();
  return *j.p == '\0';
}

}  // namespace

std::string tune_export_json() {
  std::lock_guard<std::mutex> lk(g_mu);
  const int dev = current_device();
  std::string s = "{\"advdiff_autotune\": 1, \"entries\": [";
  bool first = true;
  for (const auto& kv : g_table) {
    if (std::get<0>(kv.first) != dev || !kv.second.set) continue;
    char line[256];
    std::snprintf(line, sizeof line,
                  "%s\n  {\"kind\": %d, \"variant\": %d, \"nx\": %d, \"ny\": %d, \"nz\": %d, \"a\": %d, \"b\": %d}",
                  first ? "" : ",", std::get<1>(kv.first), std::get<2>(kv.first), std::get<3>(kv.first),
                  std::get<4>(kv.first), std::get<5>(kv.first), kv.second.a, kv.second.b);
    s += line;
    first = false;
  }
  s += first ? "]}\n" : "\n]}\n";
  return s;
}

adv_status tune_import_json(const char* text) {
  std::vector<TuneEntry> es;
  if (!parse_table(text, &es))
    return set_error(ADV_ERR_INVALID_ARG, "autotune import: not a table written by adv_autotune_export, "
                                          "or a value outside the tuner's candidates");
  {
    std::lock_guard<std::mutex> lk(g_mu);
    const int dev = current_device();
    for (const TuneEntry& e : es) g_table[Key{dev, e.kind, e.variant, e.nx, e.ny, e.nz}] = e.p;
  }
  graph_cache_clear();
  return ADV_OK;
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
  if ((st = reject_capture(s, "autotune")) != ADV_OK) return st;
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
  st = sweep(TUNE_HEAT, heat_tune_variant(*d), d->nx, d->ny, nz, cands, dflt, prep, run, reps, s, out);
  if (st != ADV_OK) return st;
  // Forward Euler can also advance two steps per launch (one pass over HBM for two updates, but
  // about twice the instructions per pass): time two tuned single-step launches against one
  // two-step launch and let adv_heat_run take the two-step kernel only where it is clearly faster.
  tune_store(TUNE_HEAT_STEPS, heat_tune_variant(*d), d->nx, d->ny, nz, TuneParams{1, 1, true});
  if (!heat2_eligible(*d, tmp.p) || !heat2_eligible(*d, tmp2.p)) return ADV_OK;
  double one_us = 0.0, two_us = 0.0;
  if ((st = prep()) != ADV_OK) return st;
  auto pair = [&]() {
    adv_status r = run();
    return r == ADV_OK ? run() : r;
  };
  if ((st = time_us(pair, reps, s, &one_us)) != ADV_OK) return st;
  HeatLaunch Ta, Tb;
  if ((st = heat2_prepare(*d, tmp2.p, &Ta)) != ADV_OK) return st;
  if ((st = heat2_prepare(*d, tmp.p, &Tb)) != ADV_OK) return st;
  auto run2 = [&]() {
    flip ^= 1;
    return flip ? heat2_launch(*d, Ta, tmp2.p, tmp.p, s) : heat2_launch(*d, Tb, tmp.p, tmp2.p, s);
  };
  if ((st = time_us(run2, reps, s, &two_us)) != ADV_OK) return st;
  if (two_us < 0.98 * one_us)
    tune_store(TUNE_HEAT_STEPS, heat_tune_variant(*d), d->nx, d->ny, nz, TuneParams{2, 1, true});
  graph_cache_clear();
  return ADV_OK;
}

adv_status adv_autotune_burgers(const adv_burgers_desc* d, const void* u, void* stream, adv_tune_result* out) {
  ADV_NVTX_RANGE("adv_autotune_burgers");
  adv_status st = burgers_validate(d);
  if (st != ADV_OK) return st;
  if (!u) return set_error(ADV_ERR_INVALID_ARG, "autotune: null buffer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if ((st = reject_capture(s, "autotune")) != ADV_OK) return st;
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
  if ((st = reject_capture(s, "autotune")) != ADV_OK) return st;
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

adv_status adv_autotune_export(char* buf, size_t capacity, size_t* length) {
  if (!length) return set_error(ADV_ERR_INVALID_ARG, "autotune export: null length");
  const std::string s = tune_export_json();
  *length = s.size() + 1;
  if (!buf) return ADV_OK;
  if (capacity < s.size() + 1) return set_error(ADV_ERR_INVALID_ARG, "autotune export: buffer too small");
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return ADV_OK;
}

adv_status adv_autotune_import(const char* json) {
  if (!json) return set_error(ADV_ERR_INVALID_ARG, "autotune import: null text");
  return tune_import_json(json);
}

}  // extern "C"
