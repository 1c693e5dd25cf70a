// driver_common.h -- shared pieces of the command-line drivers: --key=value flags, CUDA error
// exits, event timing and the reference's PrintSummary block.
#pragma once
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../../include/advdiff.h"

namespace drv {

struct Args {
  std::vector<std::string> pos;
  std::map<std::string, std::string> kv;
  std::string get(const std::string& k, const std::string& d) const {
    auto it = kv.find(k);
    return it == kv.end() ? d : it->second;
  }
  double num(const std::string& k, double d) const {
    auto it = kv.find(k);
    return it == kv.end() ? d : std::atof(it->second.c_str());
  }
};

inline Args parse(int argc, char** argv) {
  Args a;
  for (int i = 1; i < argc; ++i) {
    std::string s = argv[i];
    if (s.rfind("--", 0) == 0) {
      const size_t eq = s.find('=');
      if (eq == std::string::npos) a.kv[s.substr(2)] = "1";
      else a.kv[s.substr(2, eq - 2)] = s.substr(eq + 1);
    } else {
      a.pos.push_back(s);
    }
  }
  return a;
}

inline void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "CUDA error in %s: %s\n", what, cudaGetErrorString(e));
    std::exit(2);
  }
}
inline void check(adv_status s, const char* what) {
  if (s != ADV_OK) {
    std::fprintf(stderr, "advdiff error in %s: %s (%s)\n", what, adv_status_string(s), adv_last_error_string());
    std::exit(3);
  }
}

// --restart=path: replaces the initial state with a saved snapshot (its grid and precision must
// match the run's) and returns its step and time; without the flag, step 0 and t = t_start.
inline void restart(const Args& a, int dtype, int nx, int ny, int nz, void* host_u, size_t bytes, int64_t* step,
                    double* t, double t_start) {
  *step = 0;
  *t = t_start;
  const std::string path = a.get("restart", "");
  if (path.empty()) return;
  adv_checkpoint_header hd{};
  check(adv_checkpoint_load(path.c_str(), &hd, nullptr, 0), "restart");
  if (hd.dtype != dtype || hd.nx != nx || hd.ny != ny || hd.nz != nz) {
    std::fprintf(stderr, "restart: %s holds a %d x %d x %d %s state, the run is %d x %d x %d %s\n", path.c_str(),
                 hd.nx, hd.ny, hd.nz, hd.dtype == ADV_F32 ? "f32" : "f64", nx, ny, nz, dtype == ADV_F32 ? "f32" : "f64");
    std::exit(3);
  }
  check(adv_checkpoint_load(path.c_str(), &hd, host_u, bytes), "restart");
  *step = hd.step;
  *t = hd.t;
  std::printf("restarted from %s at step %lld, t = %.17g\n\n", path.c_str(), (long long)hd.step, hd.t);
}

// --checkpoint=path: saves the final state with its step and time.
inline void save_checkpoint(const Args& a, int dtype, int nx, int ny, int nz, int64_t step, double t,
                            const void* host_u) {
  const std::string path = a.get("checkpoint", "");
  if (path.empty()) return;
  check(adv_checkpoint_save(path.c_str(), dtype, nx, ny, nz, step, t, host_u), "checkpoint");
}

// Block layout of the reference's PrintSummary (SingleGPU/Diffusion3d_baselineCode/
// tools.cpp:185-199, SingleGPU/Burgers3d_WENO5/tools.cpp:335-350); the time is device time
// measured with CUDA events, and the rate line counts cell updates per RK stage.
inline void print_summary(const char* kernel, const char* optimization, double seconds, double h2d, double d2h,
                          double gcell_stage, const char* grid, const char* iters, double final_time) {
  std::printf("=========================== %s =======================\n", kernel);
  std::printf("Optimization                                 :  %s\n", optimization);
  std::printf("Kernel time ex. data transfers               :  %lf seconds\n", seconds);
  if (h2d >= 0) std::printf("Data transfer(s) HtD                         :  %lf seconds\n", h2d);
  if (d2h >= 0) std::printf("Data transfer(s) DtH                         :  %lf seconds\n", d2h);
  std::printf("===================================================================\n");
  std::printf("Gcell-updates/s per RK stage                 :  %lf\n", gcell_stage);
  std::printf("===================================================================\n");
  std::printf("%s\n", grid);
  std::printf("Iterations                                   :  %s\n", iters);
  if (final_time >= 0) std::printf("Final Time                                   :  %g\n", final_time);
  std::printf("===================================================================\n");
}

struct Timer {
  cudaEvent_t a, b;
  Timer() {
    check(cudaEventCreate(&a), "event");
    check(cudaEventCreate(&b), "event");
  }
  void start(cudaStream_t s) { check(cudaEventRecord(a, s), "event record"); }
  double stop(cudaStream_t s) {
    check(cudaEventRecord(b, s), "event record");
    check(cudaEventSynchronize(b), "event sync");
    float ms = 0;
    check(cudaEventElapsedTime(&ms, a, b), "event time");
    return ms * 1e-3;
  }
};

}  // namespace drv
