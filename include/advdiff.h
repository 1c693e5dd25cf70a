/*
 * advdiff.h -- native C ABI of the GB300 (sm_103a) advection-diffusion library.
 *
 * Plain C types only: raw device pointers, sizes, a cudaStream_t passed as void*. Buffers are
 * dense, x fastest, then y, then z: node (i,j,k) lives at i + nx*j + nx*ny*k, the layout of the
 * reference (SingleGPU/Diffusion3d_baselineCode/kernels.cu:113, SingleGPU/Burgers3d_WENO5/
 * kernels.cu:305). The caller owns every state buffer; the library allocates only what a plan
 * or run needs for itself (graphs, tensor maps, device scalars) and frees it on destroy.
 * Every entry point returns an adv_status and never exits the process
 * (the reference's wrappers return void and its drivers exit on CUDA errors,
 * SingleGPU/Burgers3d_WENO5/main.cpp:13-24).
 *
 * Reference interfaces this ABI replaces:
 *   adv_heat_stage / adv_heat_run   <- Call_Lu3d + Call_RK3d (SingleGPU/Diffusion3d_baselineCode/
 *                                      acoustics3d.h:57-59), Call_Lu2d + Call_RK2d
 *                                      (SingleGPU/Diffusion2d/diffusion2d.h:57-59), fused into one
 *                                      launch per stage; the host loop of main.cpp:106-122.
 *   adv_burgers_stage / _run        <- Call_Adv_x/y/z + Call_Diff_ + Call_sspRK
 *                                      (SingleGPU/Burgers3d_WENO5/Burgers.h:72-82), fused into one
 *                                      launch per SSP-RK3 stage; the host loop of main.cpp:127-150.
 *   adv_ic_* / adv_write_result_bin <- Call_Init3D / Call_Init3d / SaveBinary3D
 *                                      (SingleGPU/Diffusion3d_baselineCode/tools.cpp:59-143,
 *                                      SingleGPU/Burgers3d_WENO5/tools.cpp:241-322).
 * The reference's own extern "C" names are exported by the compatibility libraries declared
 * in advdiff_compat_heat2d.h, advdiff_compat_heat3d.h and advdiff_compat_burgers3d.h.
 */
#ifndef ADVDIFF_H
#define ADVDIFF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ADV_ABI_VERSION 3

typedef enum adv_status {
  ADV_OK = 0,
  ADV_ERR_INVALID_ARG = 1, /* bad descriptor, size, pointer alignment or enum */
  ADV_ERR_CUDA = 2,        /* a CUDA runtime/driver call failed; see adv_last_error_string() */
  ADV_ERR_TIMEOUT = 3,     /* a bounded device-side wait gave up (status word) */
  ADV_ERR_NONFINITE = 4,   /* a NaN/Inf was seen in the state (max|u| reduction) */
  ADV_ERR_CFL = 5,         /* dt rule produced a non-positive or non-finite step */
  ADV_ERR_UNSUPPORTED = 6, /* valid request this library does not implement */
  ADV_ERR_ALLOC = 7,       /* host or device allocation failed */
  ADV_ERR_BOUNDS = 8       /* checked build only: a memory index out of range (status word) */
} adv_status;

typedef enum adv_dtype { ADV_F32 = 0, ADV_F64 = 1 } adv_dtype;
typedef enum adv_time { ADV_EULER = 0, ADV_SSPRK3 = 1 } adv_time;
typedef enum adv_weno { ADV_WENO5_JS = 0, ADV_WENO5_Z = 1 } adv_weno;
typedef enum adv_lf { ADV_LF_LOCAL = 0, ADV_LF_GLOBAL = 1 } adv_lf;
typedef enum adv_bc { ADV_BC_FROZEN = 0, ADV_BC_PERIODIC = 1 } adv_bc;
/* Division of the WENO weights when the state is FP32 (one division per face side):
 * F32 = IEEE FP32 division, F64 = the division in FP64, FAST = FP32 reciprocal-based division
 * (at most 2 ulp). An FP64 state uses the reference's own operand order and its four FP64
 * divisions per side (bit-exact) with F32 or F64, and with FAST the common-denominator form:
 * one FP64 division per side, fused multiply-adds, flux differences times 1/h (a few ulps from
 * the reference's rounding). */
typedef enum adv_div { ADV_DIV_F32 = 0, ADV_DIV_F64 = 1, ADV_DIV_FAST = 2 } adv_div;
/* Burgers time-step rule. FIXED: dt = min(CFL*dx/1, 0.9/(2C sum 1/h^2)) as the reference driver
 * (SingleGPU/Burgers3d_WENO5/main.cpp:130-133); MAXU: dt = CFL*dx/max|u^n| computed on the
 * device each step (Matlab_Prototipes/InviscidBurgersNd/LFWENO5FDM3d.m:71). Both trim the last
 * step to land on tEnd and accumulate t in FP64. */
typedef enum adv_dt_rule { ADV_DT_FIXED = 0, ADV_DT_MAXU = 1 } adv_dt_rule;

/* ---------------------------------------------------------------------------- heat
 * One fused stage computes u_out = combine(u_n, u_in + dt * L(u_in)) on the updated nodes,
 * with L = kx*Sx + ky*Sy (+ kz*Sz) and per axis
 *   order 2: S = u[+1] - 2u + u[-1]                  (kernels.cu:37-64, the O2 7-pt kernel)
 *   order 4: S = -u[+2] + 16u[+1] - 30u + 16u[-1] - u[-2]  (kernels.cu:66-99, the 13-pt kernel)
 * The reference sets k = C/(12 h^2) for order 4 (main.cpp:62-64); order 2 takes k = C/h^2.
 * stage 1 (= forward Euler): u_n + dt L; stage 2: 3/4 u_n + 1/4 (u_in + dt L);
 * stage 3: (u_n + 2 (u_in + dt L)) / 3 (kernels.cu:104-142).
 * Nodes closer than `frozen` layers to any face are not updated: they are copied from u_in, or
 * written as 0 on the outermost layer when zero_boundary is set (Dirichlet u = 0).
 * The reference freezes 2 layers in 3D (kernels.cu:127) and 3 in 2D (Diffusion2d/kernels.cu:53).
 */
typedef struct adv_heat_desc {
  int32_t ndim;          /* 2 or 3 */
  int32_t nx, ny, nz;    /* nodes per axis; nz = 1 when ndim == 2 */
  int32_t dtype;         /* adv_dtype */
  int32_t order;         /* 2 or 4 */
  int32_t frozen;        /* >= order/2 */
  int32_t zero_boundary; /* 0 or 1 */
  double kx, ky, kz;     /* per-axis coefficients (kz ignored in 2D) */
  double dt;
  /* FP64 evaluation form. 0: the reference's operand order, every operation rounded on its own
   * (bit-exact with the reference's kernels built without contraction); 1: the fused
   * multiply-add pattern the FP32 state always uses (per axis O2 fma(-2, c, p1) + m1, O4
   * fma(16, far1, fma(-30, c, fma(16, near1, -near2))) - far2; L = fma(kz, Sz, fma(ky, Sy,
   * kx Sx)); stages fma(dt, L, un) | fma(0.25, fma(dt, L, uin), 0.75 un) | fma(2, fma(dt, L,
   * uin), un) / 3): six fewer FP64 operations per node on the O2 stencil, a few ulps from form
   * 0. Ignored for FP32. */
  int32_t contract;
  int32_t pad0;
} adv_heat_desc;

/* u_in and u_out must not alias; u_n may alias u_out (it is read at the written node only). */
adv_status adv_heat_stage(const adv_heat_desc* d, int stage, const void* u_in, const void* u_n,
                          void* u_out, void* stream);
/* Bytes of caller-provided workspace adv_heat_run needs: one state array for Euler, two for
 * SSP-RK3. */
adv_status adv_heat_workspace_bytes(const adv_heat_desc* d, int time_scheme, size_t* bytes);
/* nsteps time steps of the chosen scheme; the result is left in u. Asynchronous on `stream`.
 * Inside a caller's stream capture the stage launches are recorded into that capture (no graph
 * of the library's own), so the whole run can be part of the caller's graph. */
adv_status adv_heat_run(const adv_heat_desc* d, int time_scheme, int64_t nsteps, void* u,
                        void* workspace, void* stream);

/* Bytes of the fixed device scratch array behind adv_heat_run_noalloc (16 MiB). */
#define ADV_NOALLOC_SCRATCH_BYTES ((size_t)16 << 20)

/* adv_heat_run without any allocation, for callers that cannot allocate device memory: hosts
 * whose device memory is owned entirely by their own allocator (a pool that reserves the GPU's
 * memory at start-up, so a library's cudaMalloc would fail or bypass its accounting), and loops
 * that must not call cudaMalloc/cudaFree at all because those calls may synchronise the device.
 * No counterpart in the reference (its drivers cudaMalloc u, uo and Lu themselves).
 * The intermediate state lives in one file-scope __device__ array of ADV_NOALLOC_SCRATCH_BYTES
 * that every GPU loading this library holds until the process exits; the stages are launched
 * directly on `stream` (no graph, no stream, no cudaMalloc/cudaFree). A run needing more scratch
 * than adv_heat_workspace_bytes allows within that size (one state array for Euler, two for
 * SSP-RK3) is rejected with ADV_ERR_INVALID_ARG. The first call on a device (and the first after
 * the device's context was reset) looks up the array's device address and may load the module:
 * make that first call before any stream capture. All calls share the one array and it keeps the
 * last call's contents (nothing in it needs to start at zero): calls that overlap on the GPU, on
 * any streams or threads, race. */
adv_status adv_heat_run_noalloc(const adv_heat_desc* d, int time_scheme, int64_t nsteps, void* u,
                                void* stream);

/* ------------------------------------------------------------------ device-side errors
 * A kernel that cannot finish (a bounded wait for a shared-memory copy that gave up after 2 s)
 * or a time loop that meets a NaN/Inf or a non-positive dt records the first such code in a
 * per-device status word and returns; nothing traps or spins without limit. Calls that read
 * results back (adv_burgers_run/resume, adv_max_abs, adv_ensemble_run) return the word
 * themselves. The asynchronous calls (stages, adv_heat_run, adv_heat_run_noalloc, the heat-k and
 * Burgers adjoint calls) cannot: after them, adv_device_status synchronises `stream`, returns
 * the recorded code (ADV_OK if none) and clears it. This replaces the reference's checkCuda,
 * which prints and exits the process (SingleGPU/Burgers3d_WENO5/main.cpp:13-24). Called while
 * `stream` is being captured it returns ADV_ERR_UNSUPPORTED and touches nothing. */
adv_status adv_device_status(void* stream);

/* 1 in the bounds-checked build of the library (libadvdiff_checked.so: every global-memory index of
 * the stage kernels and the reference operators, and the dynamic shared-memory indices, tested
 * before use; a failed test skips the access and records ADV_ERR_BOUNDS for adv_device_status),
 * 0 in the normal build. No counterpart in the reference. */
int adv_bounds_checked(void);

/* For tests of the failure path only: one adv_heat_stage launch in which the shared-memory copy
 * of z plane `plane` is never issued, and the waits for planes give up after wait_limit_ns
 * (1e5 .. 2e9 ns). Every CTA that streams that plane then waits until its limit runs out,
 * records ADV_ERR_TIMEOUT in the status word, lets its copies already in flight land, and
 * returns; the output is left incomplete. Nothing faults or waits without limit. Takes stage 1
 * (u_n == u_in) of an FP32 3D O2 problem on the TMA load path (16-byte aligned buffer and rows);
 * ADV_ERR_UNSUPPORTED otherwise. It runs its own build of the stage kernel: the kernels every other
 * call launches carry none of this test's code. No counterpart in the reference. */
adv_status adv_test_heat_stage_withheld(const adv_heat_desc* d, int stage, const void* u_in,
                                        const void* u_n, void* u_out, int plane, uint64_t wait_limit_ns,
                                        void* stream);

/* --------------------------------------------------------------------------- Burgers
 * u_t + (u^2/2)_x + (u^2/2)_y + (u^2/2)_z = nu * Lap(u). One fused launch per SSP-RK3 stage:
 * Lax-Friedrichs split f+- = (u^2/2 +- a u)/2 with a = |u| per node (local, the reference's
 * kernels.cu:224-238) or a = max|u_in| (global); WENO5-JS (kernels.cu:92-140) or WENO5-Z
 * (kernels.cu:142-192) face fluxes along x, y, z; RHS L = -(dF)/dx - (dG)/dy - (dH)/dz
 * (+ the O4 viscous term with coefficients kx,ky,kz when nonzero, kernels.cu:444-494);
 * stage update as for heat. BC FROZEN leaves the outer 3 layers untouched (kernels.cu:518);
 * PERIODIC wraps every neighbour index. The same launch also reduces max|u_out| for the next
 * stage's Lax-Friedrichs constant and time step.
 */
typedef struct adv_burgers_desc {
  int32_t nx, ny, nz;
  int32_t dtype;  /* adv_dtype: state and flux precision */
  int32_t weno;   /* adv_weno */
  int32_t lf;     /* adv_lf */
  int32_t bc;     /* adv_bc */
  int32_t div;    /* adv_div (FP32 state only) */
  int32_t bug_b2; /* 1: add the viscous term twice on slabs 16..18 as the reference does */
  int32_t pad0;
  double dx, dy, dz;
  double kx, ky, kz; /* viscous O4 coefficients C/(12 h^2); all 0 = inviscid */
} adv_burgers_desc;

/* One stage. alpha is the global Lax-Friedrichs constant (ignored for local LF).
 * maxabs_out, if non-NULL, is a device float (FP32 state) or double (FP64 state) that receives
 * max(|u_out|) via atomicMax; the caller zeroes it first. */
adv_status adv_burgers_stage(const adv_burgers_desc* d, int stage, const void* u_in,
                             const void* u_n, void* u_out, double dt, double alpha,
                             void* maxabs_out, void* stream);
adv_status adv_burgers_workspace_bytes(const adv_burgers_desc* d, size_t* bytes);
/* Full time loop to tEnd (at most max_steps steps). dt and the global-LF constant are computed
 * on the device; the loop runs as one CUDA graph (a while-conditional node when the driver
 * supports it, else fixed-size predicated chunks). C is the viscous coefficient used only by
 * ADV_DT_FIXED's diffusive bound (0 drops it). t_out / steps_out may be NULL. Synchronises the
 * stream to read t and the step count back; called while the stream is being captured it
 * returns ADV_ERR_UNSUPPORTED and leaves the stream and the capture untouched (record
 * adv_burgers_stage calls instead). The same holds for adv_burgers_resume, adv_max_abs,
 * adv_ensemble_run and the autotuner. */
adv_status adv_burgers_run(const adv_burgers_desc* d, void* u, void* workspace, double tEnd,
                           double cfl, int dt_rule, double C, int64_t max_steps, double* t_out,
                           int64_t* steps_out, void* stream);
/* adv_burgers_run continued from a saved state (adv_checkpoint_save): the time sum starts at t0
 * and the step count at step0, so a run stopped after step0 steps (max_steps) and resumed ends
 * bit for bit where the uninterrupted run ends. (A run stopped at a tEnd between steps took a
 * shortened last step there, so it is a different run.) max_steps, t_out and steps_out count
 * from the start of the whole run. */
adv_status adv_burgers_resume(const adv_burgers_desc* d, void* u, void* workspace, double t0,
                              int64_t step0, double tEnd, double cfl, int dt_rule, double C,
                              int64_t max_steps, double* t_out, int64_t* steps_out, void* stream);

/* ----------------------------------------------------------------- WENO7 Burgers (prototype)
 * The reference's seventh-order prototype solver of u_t + (u^2/2)_x + (u^2/2)_y (+ (u^2/2)_z) = 0
 * (Matlab_Prototipes/InviscidBurgersNd/WENO7resAdv_{X,Y,Z}.m, LFWENO7FDM{2,3}d.m:65-104): local
 * Lax-Friedrichs split, every line extended past its ends by copies of its end values with the
 * face left of its first node taken as 0, the Balsara-Shu WENO7 reconstruction with the
 * prototype's integer smoothness indicators, the residuals summed in axis order, and the
 * Carpenter-Kennedy five-stage fourth-order 2N-storage Runge-Kutta step with dt = CFL dx /
 * max|u| trimmed to land on tEnd. An FP64 state reproduces the prototypes' arithmetic operand for
 * operand; an FP32 state evaluates the same scheme in a faster form of its own (its weights from
 * the smallest eps + beta_k, reciprocal-based divisions of at most 2 ulp), within 5e-6 relative L2
 * of the FP64 residual. 2D (nz == 1) and 3D grids, node (i,j,k) at i + nx*j + nx*ny*k. */
typedef struct adv_weno7_desc {
  int32_t nx, ny, nz;
  int32_t dtype; /* adv_dtype */
  double dx, dy, dz;
} adv_weno7_desc;

/* Workspace of adv_weno7_rhs / adv_weno7_run: four state arrays and a loop state. */
adv_status adv_weno7_workspace_bytes(const adv_weno7_desc* d, size_t* bytes);
/* L = the summed prototype residuals (df/dx + df/dy (+ df/dz), the sign of the prototypes' res).
 * Asynchronous. */
adv_status adv_weno7_rhs(const adv_weno7_desc* d, const void* u, void* L, void* workspace, void* stream);
/* The prototype's time loop to tEnd (at most max_steps steps) in place on u, as one CUDA graph with
 * a device-driven loop. Synchronises the stream (reads t and the step count back); inside a stream
 * capture it returns ADV_ERR_UNSUPPORTED. */
adv_status adv_weno7_run(const adv_weno7_desc* d, void* u, void* workspace, double tEnd, double cfl,
                         int64_t max_steps, double* t_out, int64_t* steps_out, void* stream);

/* ------------------------------------------- heat with a diffusivity field k(x), and its adjoint
 * u_t = div(k grad u) on a 3D node grid: conservative 7-point form with arithmetic face averages
 * k_{i+1/2} = (k_i + k_{i+1})/2, forward Euler, c_a = dt / h_a^2:
 *   u'_i = u_i + sum_a c_a [k_{i+1/2}(u_{i+1} - u_i) - k_{i-1/2}(u_i - u_{i-1})]   (interior)
 * The outermost layer is frozen (held, or set to 0 with zero_boundary). No counterpart in the
 * reference (its diffusivity is one constant, SingleGPU/Diffusion3d_baselineCode/main.cpp:58-61).
 * The adjoint step is the exact transpose of one step: given lam' = dJ/du^{n+1} and u^n it
 * writes lam = dJ/du^n and adds this step's dJ/dk into grad_k. */
typedef struct adv_heatk_desc {
  int32_t nx, ny, nz;
  int32_t dtype;          /* adv_dtype */
  int32_t zero_boundary;  /* 0 or 1 */
  int32_t pad0;
  double cx, cy, cz;      /* dt / h_a^2 */
} adv_heatk_desc;

adv_status adv_heatk_step(const adv_heatk_desc* d, const void* k, const void* u_in, void* u_out,
                          void* stream);
adv_status adv_heatk_adjoint_step(const adv_heatk_desc* d, const void* k, const void* u_n,
                                  const void* lam_next, void* lam_out, void* grad_k, void* stream);
/* Checkpointing: the forward run stores u every `interval` steps (ceil(nsteps/interval) arrays in
 * ckpt; each stored state is written there by the step that makes it); the backward run
 * recomputes each interval from its checkpoint into `work` (interval arrays) and sweeps the
 * adjoint through it. interval ~ sqrt(nsteps) keeps memory at ~2 sqrt(nsteps) arrays; interval 1
 * keeps every state (nsteps arrays) and the backward run recomputes nothing. Sizes in bytes. */
adv_status adv_heatk_checkpoint_bytes(const adv_heatk_desc* d, int64_t nsteps, int64_t interval,
                                      size_t* ckpt_bytes, size_t* work_bytes);
/* nsteps steps in place on u; ckpt may be NULL (no checkpoints kept). With checkpoints, the run
 * also leaves the states of its last checkpoint interval (u^{n0+1} .. u^{nsteps-1}) in work, where
 * adv_heatk_backward would recompute them. */
adv_status adv_heatk_forward(const adv_heatk_desc* d, const void* k, void* u, int64_t nsteps,
                             int64_t interval, void* ckpt, void* work, void* stream);
/* lam: in dJ/du at step nsteps, out dJ/du at step 0. grad_k += dJ/dk. flags:
 * ADV_HEATK_LAST_INTERVAL_IN_WORK when work still holds what adv_heatk_forward left there (the
 * same nsteps, interval and ckpt, nothing written to work since): the last interval is then not
 * recomputed. */
#define ADV_HEATK_LAST_INTERVAL_IN_WORK 1
adv_status adv_heatk_backward(const adv_heatk_desc* d, const void* k, int64_t nsteps,
                              int64_t interval, const void* ckpt, void* lam, void* grad_k,
                              void* work, int flags, void* stream);

/* --------------------------------------------------------------- Burgers discrete adjoint
 * Exact transpose of the fixed-dt SSP-RK3 step of the periodic, local Lax-Friedrichs, inviscid
 * scheme (WENO5-JS or WENO5-Z; FP32 or FP64 state; other schemes return ADV_ERR_UNSUPPORTED).
 * No counterpart in the reference. adv_burgers_adjoint_step turns lam = dJ/du^{n+1} into
 * dJ/du^n given the step's stage inputs u^n, u1, u2; `work` holds 3 arrays. The forward run
 * stores u every `interval` steps; the backward run recomputes each interval (its stage inputs)
 * from the checkpoint and sweeps the adjoint back through it. */
adv_status adv_burgers_adjoint_step(const adv_burgers_desc* d, const void* u_n, const void* u1,
                                    const void* u2, double dt, void* lam, void* work, void* stream);
/* ckpt: ceil(nsteps/interval) arrays; work: 3*interval + 2 arrays (enough for both runs). */
adv_status adv_burgers_checkpoint_bytes(const adv_burgers_desc* d, int64_t nsteps, int64_t interval,
                                        size_t* ckpt_bytes, size_t* work_bytes);
/* nsteps fixed-dt steps in place on u; ckpt may be NULL. With checkpoints, the run also leaves
 * the stage inputs of its last checkpoint interval in work, where adv_burgers_backward would
 * recompute them (interval >= nsteps: every stage input of the run, 3*nsteps - 1 arrays). */
adv_status adv_burgers_forward(const adv_burgers_desc* d, void* u, double dt, int64_t nsteps,
                               int64_t interval, void* ckpt, void* work, void* stream);
/* lam: in dJ/du at step nsteps, out dJ/du at step 0. flags: ADV_BURGERS_LAST_INTERVAL_IN_WORK
 * when work still holds what adv_burgers_forward left there (the same nsteps, interval, dt and
 * ckpt, nothing written to work since): the last interval is then not recomputed. */
#define ADV_BURGERS_LAST_INTERVAL_IN_WORK 1
adv_status adv_burgers_backward(const adv_burgers_desc* d, double dt, int64_t nsteps,
                                int64_t interval, const void* ckpt, void* lam, void* work,
                                int flags, void* stream);

/* ------------------------------------------------------------------ batched ensembles
 * Many independent 3D problems of uneven size and coefficients advanced together. No counterpart
 * in the reference (its drivers run one problem per process). Each stage of all heat members is
 * ONE launch over every member's (tile, z-plane) units, each SSP-RK3 stage of all Burgers
 * members likewise, and a whole run is one CUDA graph holding the heat and the Burgers time
 * loops as two concurrent device-driven while-loops (dt, the Lax-Friedrichs constants and each
 * Burgers member's stop test are computed on the device, per member).
 * Heat members share dtype, order and the time scheme (given at create); ndim must be 3; sizes,
 * coefficients, dt, frozen layers and boundary handling are per member. Burgers members share
 * dtype, weno, div and whether the viscous term is present; sizes, spacing, lf, bc, bug_b2,
 * tEnd, CFL and the dt rule are per member. Results equal the per-member adv_heat_run /
 * adv_burgers_run bit for bit. Each member's state stays in its caller-owned buffer u; `work` is
 * caller-owned scratch of adv_heat_workspace_bytes / adv_burgers_workspace_bytes bytes.
 * Buffers must not overlap between members. The plan allocates its device tables, loop states
 * and graph at create (runs allocate nothing) and frees them at destroy. */
typedef struct adv_heat_member {
  adv_heat_desc desc;
  void* u;
  void* work;
} adv_heat_member;

typedef struct adv_burgers_member {
  adv_burgers_desc desc;
  void* u;
  void* work;
  double tEnd, cfl;
  int32_t dt_rule; /* adv_dt_rule */
  int32_t pad0;
  double C;          /* viscous coefficient for ADV_DT_FIXED's diffusive bound (0 drops it) */
  int64_t max_steps; /* per-member step limit */
} adv_burgers_member;

typedef struct adv_ensemble adv_ensemble;

/* Either count may be 0. heat_time_scheme: adv_time. The device current at create is the
 * plan's device. */
adv_status adv_ensemble_create(const adv_heat_member* heat, int n_heat, int heat_time_scheme,
                               const adv_burgers_member* burgers, int n_burgers, adv_ensemble** out);
/* heat_steps steps of every heat member and every Burgers member run to its tEnd (at most its
 * max_steps), from the current contents of the members' u. ADV_ENSEMBLE_DIRECT launches the
 * same kernels from the host instead of the graph (for comparison; Burgers then reads a stop
 * flag back every 8 steps). Synchronises the stream. */
#define ADV_ENSEMBLE_DIRECT 1
adv_status adv_ensemble_run(adv_ensemble* e, int64_t heat_steps, int flags, void* stream);
/* Time reached and steps taken by Burgers member i in the last run. */
adv_status adv_ensemble_burgers_result(const adv_ensemble* e, int i, double* t, int64_t* steps);
/* Units (tile-planes) per heat / Burgers stage launch and the CTAs of each launch (any pointer
 * may be NULL). */
adv_status adv_ensemble_shape(const adv_ensemble* e, int64_t* heat_units, int* heat_ctas,
                              int64_t* burgers_units, int* burgers_ctas);
adv_status adv_ensemble_destroy(adv_ensemble* e);

/* ------------------------------------------------------------------------- autotuner
 * Times the candidate launch shapes of a problem on the caller's data (out of place: the state is
 * not modified; a temporary buffer is allocated and freed on the stream) and keeps the fastest for
 * every later call on this device with the same problem shape, for the life of the process. No
 * counterpart in the reference (its drivers take the block sizes on the command line).
 *   heat / Burgers stages: param_a = CTAs per SM (up to the kernel's occupancy), param_b =
 *     minimum z planes per CTA share (the z-halo re-reads vs tail balance trade-off);
 *   heat with k(x), step and adjoint kernels: param_a = block height, param_b = z planes per CTA.
 * adv_autotune_heat also times, for FP32 3D O2 problems with rows of whole 16-byte vectors, one
 * launch of the two-step kernel (two forward-Euler steps per pass over HBM) against two tuned
 * single-step launches; adv_heat_run's forward-Euler loop takes two-step launches for that problem
 * only if they were more than 2% faster (table kind 5, a = steps per launch). Its result (out)
 * describes the single-step shape.
 * Synchronises the stream. */
typedef struct adv_tune_result {
  int32_t kind;
  int32_t param_a, param_b;
  int32_t candidates;
  double best_us;     /* mean time per launch of the chosen shape */
  double default_us;  /* the same for the untuned default shape */
} adv_tune_result;

adv_status adv_autotune_heat(const adv_heat_desc* d, const void* u, void* stream, adv_tune_result* out);
adv_status adv_autotune_burgers(const adv_burgers_desc* d, const void* u, void* stream,
                                adv_tune_result* out);
adv_status adv_autotune_heatk(const adv_heatk_desc* d, const void* k, const void* u, void* stream,
                              adv_tune_result* out_step, adv_tune_result* out_adjoint);
/* Forgets every tuned shape (launches return to the defaults). */
adv_status adv_autotune_clear(void);
/* The tuned shapes of the current device as JSON text, to keep them between processes:
 * {"advdiff_autotune": 1, "entries": [{"kind": .., "variant": .., "nx": .., "ny": .., "nz": ..,
 * "a": .., "b": ..}, ...]}. *length receives the size including the terminating NUL; with
 * buf == NULL only the size is returned. */
adv_status adv_autotune_export(char* buf, size_t capacity, size_t* length);
/* Loads a table written by adv_autotune_export for the current device (entries replace tuned
 * shapes of the same problems). Rejects, without loading anything, text in any other form and
 * values outside the tuner's own candidates (ADV_ERR_INVALID_ARG). */
adv_status adv_autotune_import(const char* json);

/* ------------------------------------------------------------------ reductions
 * max|u| over n values into *out (host double). Synchronises the stream. */
adv_status adv_max_abs(int dtype, const void* u, int64_t n, double* out, void* stream);

/* ----------------------------------------------------------- initial conditions (host)
 * Seeded inputs use Philox4x32-10 (counter-based) so every consumer regenerates them exactly. */
/* Reference heat IC 3 (tools.cpp:128-139): exp(-|x-5|^2/(4*0.1)) at nodes (i dx, j dy, k dz),
 * faces zeroed; ndim 2 or 3. */
adv_status adv_ic_heat_ref(int ndim, int nx, int ny, int nz, double dx, double dy, double dz,
                           double* u);
/* 2D: Gaussian bump exp(-((x-.5)^2+(y-.5)^2)/0.01) + N(0, sigma^2) noise on [0,1]^2, edges 0. */
adv_status adv_ic_heat2d_gauss_noise(int nx, int ny, uint32_t seed, double sigma, double* u);
/* 3D: sum of nblobs Gaussians, centres U[0.2,0.8]^3, widths U[0.02,0.08], on [0,1]^3, faces 0. */
adv_status adv_ic_heat3d_blobs(int nx, int ny, int nz, uint32_t seed, int nblobs, double* u);
/* Burgers: 0.5 + sum of nmodes a cos(pi n.x + phi), |n| <= 4, a ~ U[0,amax], on the periodic
 * cell centres of [0,L)^3. */
adv_status adv_ic_burgers_fourier(int nx, int ny, int nz, double L, uint32_t seed, int nmodes,
                                  double amax, double* u);
/* Reference Burgers IC 3 (tools.cpp:126-137): exp(-|x-1|^2/0.1) at (i dx, j dy, k dz). */
adv_status adv_ic_burgers_ref(int nx, int ny, int nz, double dx, double dy, double dz, double* u);
/* The reference's 2D Burgers IC 3 (MultiGPU/Burgers2d_Baseline/Tools.c:108-119): exp(-(x^2+y^2)/0.1)
 * with x = (0.5 (nx-1) - i) dx, y = (0.5 (ny-1) - j) dy, zero on the outer ring of nodes. */
adv_status adv_ic_burgers_ref2d(int nx, int ny, double dx, double dy, double* u);

/* ---------------------------------------------------------------------- output (host)
 * result.bin as the reference writes it: float32, x fastest, no header
 * (SingleGPU/Diffusion3d_baselineCode/tools.cpp:59-87). */
adv_status adv_write_result_bin(const char* path, int dtype, const void* host_u, int64_t n);
/* Reads a result.bin / initial.bin of exactly n float32 values into doubles (the file size must
 * match). */
adv_status adv_read_result_bin(const char* path, int64_t n, double* host_u);
/* The reference's multi-GPU programs write their whole z-decomposed array, RADIUS ghost slabs at
 * each z end included: nx*ny*(nz + 2*radius) values (MultiGPU/Burgers3d_Baseline/main.c:65,79,
 * 355; RADIUS 3 for WENO5). Strip keeps the nz interior slabs; pad writes the ghosts as copies of
 * the periodic neighbours (periodic != 0) or zeros. */
adv_status adv_strip_ghost_slabs(int nx, int ny, int nz, int radius, const double* ghosted,
                                 double* interior);
adv_status adv_pad_ghost_slabs(int nx, int ny, int nz, int radius, int periodic,
                               const double* interior, double* ghosted);

/* State snapshot for resuming a run (no counterpart in the reference, which keeps no restart
 * state): a 128-byte header (magic "ADVSTATE", version 1, dtype, nx, ny, nz, step, t, payload
 * size, CRC-32 of the payload and of the header) then the state in its own precision, x
 * fastest. Saved through a temporary file and a rename; loading checks both CRCs and rejects a
 * truncated, altered or inconsistent file. host_u NULL: read the header only. */
typedef struct adv_checkpoint_header {
  int32_t version, dtype;
  int32_t nx, ny, nz, pad0;
  int64_t step;
  double t;
  uint64_t payload_bytes;
  uint32_t payload_crc32, pad1;
} adv_checkpoint_header;
adv_status adv_checkpoint_save(const char* path, int dtype, int nx, int ny, int nz, int64_t step,
                               double t, const void* host_u);
adv_status adv_checkpoint_load(const char* path, adv_checkpoint_header* hdr, void* host_u,
                               size_t capacity_bytes);
/* CRC-32 (IEEE 802.3 polynomial, as zlib) of n bytes. */
uint32_t adv_crc32(const void* data, size_t n);

/* ------------------------------------------------------------------------- misc */
const char* adv_last_error_string(void);
const char* adv_status_string(adv_status s);
int adv_abi_version(void);
/* Kernels this library launched since load (for launch-count accounting). */
int64_t adv_kernel_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* ADVDIFF_H */
