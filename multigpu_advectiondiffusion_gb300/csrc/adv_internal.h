// adv_internal.h -- declarations shared by the library's translation units (not installed).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/advdiff.h"

namespace adv {

// Records a message for adv_last_error_string() and returns `s`.
adv_status set_error(adv_status s, const std::string& msg);
adv_status cuda_error(cudaError_t e, const char* what);
void count_launches(int64_t n);

#define ADV_CUDA_TRY(call)                                    \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ::adv::cuda_error(e_, #call); \
  } while (0)

// Device properties used for launch sizing, cached per device.
struct DeviceInfo {
  int device = -1;
  int sms = 0;
  int cc_major = 0, cc_minor = 0;
  size_t smem_optin = 0;
};
adv_status device_info(DeviceInfo* out);

// cuTensorMapEncodeTiled resolved through the runtime (no -lcuda link needed).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled_fn();

// True while `s` is being captured into a CUDA graph.
bool stream_capturing(cudaStream_t s);
// ADV_ERR_UNSUPPORTED for a call that reads results back to the host (and so synchronises `s`)
// while `s` is being captured; the stream and the caller's capture are left untouched.
adv_status reject_capture(cudaStream_t s, const char* what);

// Device status word (per device): 0 = OK, else an adv_status raised by a kernel. Reading it
// synchronises `s`; a nonzero word is returned as the status and cleared.
adv_status read_and_clear_device_status(cudaStream_t s);
int* device_status_ptr();

// ------------------------------------------------------------------ launch-shape tuning
// Parameters picked by the autotuner (autotune.cu) per device and problem; `set` is false when the
// problem was never tuned (launchers then use their defaults). Kinds and parameters:
//   TUNE_HEAT, TUNE_BURGERS: a = CTAs per SM (<= occupancy), b = minimum planes per CTA share
//   TUNE_HEATK_STEP, TUNE_HEATK_ADJ: a = block height (threads in y), b = z planes per CTA
//   TUNE_HEAT_STEPS: a = forward-Euler time steps per launch of adv_heat_run (1, or 2 with the
//     two-step kernel where it measured faster), b = 1
enum TuneKind { TUNE_HEAT = 1, TUNE_BURGERS = 2, TUNE_HEATK_STEP = 3, TUNE_HEATK_ADJ = 4, TUNE_HEAT_STEPS = 5 };
struct TuneParams {
  int a = 0, b = 0;
  bool set = false;
};
TuneParams tune_lookup(int kind, int variant, int nx, int ny, int nz);
void tune_store(int kind, int variant, int nx, int ny, int nz, TuneParams p);
void tune_clear();
void graph_cache_clear();  // cached CUDA graphs hold launch shapes: drop them when tuning changes

// ------------------------------------------------------------------ heat launchers
// "No plane withheld": below every plane a stream can visit (halo planes reach z = -2).
constexpr int kNoWithheldPlane = -2147483647 - 1;
struct HeatLaunch {
  // resolved per plan: whether the TMA path applies and the chosen z-chunk
  bool tma = false;
  int occ = 0;                   // resident CTAs per SM of the stage kernel (before any tuning cap)
  int rows = 2;                  // rows per thread
  int warps = 8;                 // warps per CTA
  int lanes = 32;                // lanes per row (16: two rows per warp); tile lanes*vector x (32*warps/lanes)*rows
  int tiles_x = 0, tiles_y = 0;  // x-y tiles; the grid is one wave of CTAs sharing the tile-planes
  dim3 grid, block;
  size_t smem = 0;
  CUtensorMap tmap_in;  // tensor map of u_in (re-encoded when the pointer changes)
  // failure-path testing only (adv_test_heat_stage_withheld): a z plane whose copy is never
  // issued (kNoWithheldPlane: none -- negative planes are real halo planes), and the wait limit
  // for planes (0: the normal limit)
  int withheld_plane = kNoWithheldPlane;
  unsigned long long wait_limit_ns = 0;
};
// rows: rows per thread of the stage kernel (2 or 4), lanes: lanes per row (32 or 16); 0 = the
// library's choice.
adv_status heat_prepare(const adv_heat_desc& d, const void* u_in, HeatLaunch* L, int rows = 0, int lanes = 0);
// Lanes per row of the 4-row FP32 tile for rows of nx nodes: 16 (64-wide tiles) where 128-wide
// tiles leave clearly more lanes idle, else 32.
int heat_row_lanes(int nx);
// 2D forward Euler, up to heat2d_multi_steps() steps per launch (heat2d_multi.cu); in != out.
int heat2d_multi_steps();
adv_status heat2d_multi_launch(const adv_heat_desc& d, const void* in, void* out, int steps, cudaStream_t s);
adv_status heat_launch(const adv_heat_desc& d, const HeatLaunch& L, int stage, const void* u_in,
                       const void* u_n, void* u_out, cudaStream_t s);
adv_status heat_validate(const adv_heat_desc* d);
// One stage-1 launch of the failure-path test's kernel variant (FP32 3D O2, TMA, L's withheld plane
// and wait limit); ADV_ERR_UNSUPPORTED for other problems.
adv_status heat_launch_test_hook(const adv_heat_desc& d, const HeatLaunch& L, const void* u_in, void* u_out,
                                 cudaStream_t s);
// Two forward-Euler steps per launch (FP32 3D O2, rows of whole 16-byte vectors, TMA path):
// u_out = E(E(u_in)), bit for bit two heat_launch stage-1 steps.
bool heat2_eligible(const adv_heat_desc& d, const void* u_in);
adv_status heat2_prepare(const adv_heat_desc& d, const void* u_in, HeatLaunch* L);
adv_status heat2_launch(const adv_heat_desc& d, const HeatLaunch& L, const void* u_in, void* u_out, cudaStream_t s);
int heat_tune_variant(const adv_heat_desc& d);

// --------------------------------------------------------------- Burgers launchers
struct BurgersLaunch {
  bool tma = false;
  int occ = 0;  // resident CTAs per SM of the stage kernel (before any tuning cap)
  int tiles_x = 0, tiles_y = 0;  // 32 x 16 column tiles; the grid is one wave sharing the tile-planes
  dim3 grid, block;
  size_t smem = 0;
  CUtensorMap tmap_in;
};
adv_status burgers_validate(const adv_burgers_desc* d);
int burgers_tune_variant(const adv_burgers_desc& d);
adv_status burgers_prepare(const adv_burgers_desc& d, const void* u_in, BurgersLaunch* L);
// Stage launch arguments. The Lax-Friedrichs constant and dt come from the host values unless
// a device source is given (used by the graph-resident time loop).
struct BurgersStageArgs {
  int stage;
  const void* u_in;
  const void* u_n;
  void* u_out;
  double dt_host;
  double alpha_host;
  const double* dt_dev;     // nullable: dt as FP64
  const double* alpha_dev;  // nullable: LF constant as FP64
  const void* alpha_key;    // nullable: max|u| key of the previous stage (FP32/FP64 bits)
  void* maxabs_key;         // nullable: accumulator key for max|u_out|
  const int* active;        // nullable: kernel returns at once when *active == 0
};
adv_status burgers_launch(const adv_burgers_desc& d, const BurgersLaunch& L,
                          const BurgersStageArgs& a, cudaStream_t s);

// Loop-control state for adv_burgers_run (device resident; see api_device.cu).
struct BurgersLoopState {
  double t, tEnd, cfl, dx, dt_fixed, dt, alpha0;
  int64_t step, max_steps;
  int dt_rule, active;
  unsigned maxbits[3];              // rotating FP32 max|u| accumulators (stage s writes s % 3)
  unsigned long long maxbits64[3];  // the same for FP64 state
};
adv_status burgers_loop_begin_step(BurgersLoopState* st, int dtype, unsigned long long cond_handle,
                                   int use_cond, cudaStream_t s);
adv_status burgers_loop_begin_step_batch(BurgersLoopState* st, int n, int dtype, unsigned long long cond_handle,
                                         int use_cond, int* any_more, cudaStream_t s);
// The initial loop state of one run (t = 0, the fixed dt of ADV_DT_FIXED, slot-0 key cleared).
BurgersLoopState burgers_loop_state(const adv_burgers_desc& d, double tEnd, double cfl, int dt_rule, double C,
                                    int64_t max_steps);
adv_status max_abs_launch(int dtype, const void* u, int64_t n, void* accum_bits, cudaStream_t s);
// One iteration of a device-counted loop (see api_device.cu).
adv_status loop_tick(int64_t* remaining, int* active, unsigned long long cond_handle, int use_cond, cudaStream_t s);

}  // namespace adv
