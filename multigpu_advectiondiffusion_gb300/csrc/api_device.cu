// api_device.cu -- device-side pieces shared by the API: the status word, the max|u|
// reduction and the single-thread kernels that drive the Burgers time loop from the device
// (dt rule, t accumulation, loop condition), so a whole run is one CUDA graph with no host
// round trip per step.
#include <cuda_runtime.h>

#include <limits>

#include "adv_device.cuh"
#include "adv_internal.h"

namespace adv {

__device__ int g_status_word[1];

int* device_status_ptr() {
  // The address of a __device__ symbol is per device; resolve it each call (cheap) so the
  // pointer always belongs to the current device.
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_status_word) != cudaSuccess) return nullptr;
  return static_cast<int*>(p);
}

adv_status read_and_clear_device_status(cudaStream_t s) {
  int* p = device_status_ptr();
  if (!p) return set_error(ADV_ERR_CUDA, "status word unavailable");
  int v = 0;
  ADV_CUDA_TRY(cudaMemcpyAsync(&v, p, sizeof(int), cudaMemcpyDeviceToHost, s));
  ADV_CUDA_TRY(cudaStreamSynchronize(s));
  if (v != 0) {
    const int zero = 0;
    ADV_CUDA_TRY(cudaMemcpy(p, &zero, sizeof(int), cudaMemcpyHostToDevice));
    return set_error(static_cast<adv_status>(v), "device kernel reported an error");
  }
  return ADV_OK;
}

// ------------------------------------------------------------------- max|u| reduction
// Grid-stride: per-thread max of |u| keys, warp max with a reduction instruction, one
// atomicMax per warp into the caller's key (bits of a non-negative float/double).
template <class T>
__global__ void __launch_bounds__(256) max_abs_kernel(const T* __restrict__ u, int64_t n,
                                                      typename KeyOf<T>::type* accum) {
  using K = typename KeyOf<T>::type;
  K m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const K k = abs_key(u[i]);
    m = k > m ? k : m;
  }
  m = warp_max(m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(accum, m);
}

adv_status max_abs_launch(int dtype, const void* u, int64_t n, void* accum_bits, cudaStream_t s) {
  DeviceInfo di;
  adv_status st = device_info(&di);
  if (st != ADV_OK) return st;
  const int64_t blocks_needed = (n + 255) / 256;
  const int blocks = (int)std::min<int64_t>(std::max<int64_t>(blocks_needed, 1), (int64_t)di.sms * 8);
  if (dtype == ADV_F32)
    max_abs_kernel<float><<<blocks, 256, 0, s>>>(static_cast<const float*>(u), n, static_cast<unsigned*>(accum_bits));
  else
    max_abs_kernel<double><<<blocks, 256, 0, s>>>(static_cast<const double*>(u), n,
                                                  static_cast<unsigned long long*>(accum_bits));
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}

// ------------------------------------------------------------- Burgers loop control
// Start of a step of one run: max|u^n| from accumulator slot 0 sets dt (rule MAXU) and the
// stage-1 Lax-Friedrichs constant; the dt is trimmed to land on tEnd and t advances in FP64, in
// the order of SingleGPU/Burgers3d_WENO5/main.cpp:130-136. The accumulators for the three
// stages are cleared. A non-finite max|u| or dt stops the run and records the error in the
// status word. Returns whether another step follows this one.
__device__ int burgers_begin_step_one(BurgersLoopState* st, int dtype, int* status) {
  double m;
  if (dtype == ADV_F32) m = (double)key_to_value(st->maxbits[0]);
  else m = key_to_value(st->maxbits64[0]);
  int active = st->active;
  if (active && (st->t >= st->tEnd || st->step >= st->max_steps)) active = 0;
  if (active && !isfinite(m)) {
    raise_status(status, 4 /* ADV_ERR_NONFINITE */);
    active = 0;
  }
  double dt = 0.0;
  if (active) {
    dt = (st->dt_rule == 1) ? st->cfl * st->dx / m : st->dt_fixed;
    if (!(dt > 0.0) || !isfinite(dt)) {
      raise_status(status, 5 /* ADV_ERR_CFL */);
      active = 0;
    }
  }
  if (active) {
    if ((st->t + dt) > st->tEnd) dt = st->tEnd - st->t;
    st->t += dt;
    st->step += 1;
    st->dt = dt;
    st->alpha0 = m;
  }
  st->active = active;
  st->maxbits[1] = 0u; st->maxbits[2] = 0u;
  st->maxbits64[1] = 0ull; st->maxbits64[2] = 0ull;
  if (active) { st->maxbits[0] = 0u; st->maxbits64[0] = 0ull; }
  return active && st->t < st->tEnd && st->step < st->max_steps;
}

// Initial loop state of one run (host).
BurgersLoopState burgers_loop_state(const adv_burgers_desc& d, double tEnd, double cfl, int dt_rule, double C,
                                    int64_t max_steps) {
  BurgersLoopState h{};
  h.t = 0.0;
  h.tEnd = tEnd;
  h.cfl = cfl;
  h.dx = d.dx;
  const double dt1 = cfl * d.dx / 1.0;
  const double iz = d.nz == 1 ? 0.0 : 1 / d.dz / d.dz;  // a 2D grid has no z term
  const double dt2 = C > 0 ? 1. / (2 * C * (1 / d.dx / d.dx + 1 / d.dy / d.dy + iz)) * 0.9
                           : std::numeric_limits<double>::infinity();
  h.dt_fixed = dt1 < dt2 ? dt1 : dt2;
  h.step = 0;
  h.max_steps = max_steps;
  h.dt_rule = dt_rule;
  h.active = 1;
  return h;
}

// One run. The loop condition for the enclosing while-node is set here (the body runs to
// completion, then the condition is evaluated).
__global__ void burgers_begin_step_kernel(BurgersLoopState* st, int dtype, int* status,
                                          cudaGraphConditionalHandle cond, int use_cond) {
  const int more = burgers_begin_step_one(st, dtype, status);
  if (use_cond) cudaGraphSetConditional(cond, more ? 1u : 0u);
}

adv_status burgers_loop_begin_step(BurgersLoopState* st, int dtype, unsigned long long cond_handle, int use_cond,
                                   cudaStream_t s) {
  burgers_begin_step_kernel<<<1, 1, 0, s>>>(st, dtype, device_status_ptr(),
                                            static_cast<cudaGraphConditionalHandle>(cond_handle), use_cond);
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}

// Many runs (an ensemble's Burgers members), one thread each; the loop goes on while any run
// has another step. *any_more (if given) receives the same flag for host-driven loops.
__global__ void __launch_bounds__(256) burgers_begin_step_batch_kernel(BurgersLoopState* st, int n, int dtype,
                                                                       int* status, cudaGraphConditionalHandle cond,
                                                                       int use_cond, int* any_more) {
  int more = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) more |= burgers_begin_step_one(&st[i], dtype, status);
  more = __syncthreads_or(more);
  if (threadIdx.x == 0) {
    if (use_cond) cudaGraphSetConditional(cond, more ? 1u : 0u);
    if (any_more) *any_more = more;
  }
}

adv_status burgers_loop_begin_step_batch(BurgersLoopState* st, int n, int dtype, unsigned long long cond_handle,
                                         int use_cond, int* any_more, cudaStream_t s) {
  burgers_begin_step_batch_kernel<<<1, 256, 0, s>>>(st, n, dtype, device_status_ptr(),
                                                    static_cast<cudaGraphConditionalHandle>(cond_handle), use_cond,
                                                    any_more);
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}

// ---------------------------------------------------------- counted device loops
// One iteration of a loop of *remaining iterations: *active tells this iteration's kernels
// whether to work, and the while-node goes on while iterations remain.
__global__ void loop_tick_kernel(int64_t* remaining, int* active, cudaGraphConditionalHandle cond, int use_cond) {
  const int64_t r = *remaining;
  const int a = r > 0 ? 1 : 0;
  if (a) *remaining = r - 1;
  *active = a;
  if (use_cond) cudaGraphSetConditional(cond, (a && r > 1) ? 1u : 0u);
}

adv_status loop_tick(int64_t* remaining, int* active, unsigned long long cond_handle, int use_cond, cudaStream_t s) {
  loop_tick_kernel<<<1, 1, 0, s>>>(remaining, active, static_cast<cudaGraphConditionalHandle>(cond_handle), use_cond);
  ADV_CUDA_TRY(cudaGetLastError());
  count_launches(1);
  return ADV_OK;
}

}  // namespace adv
