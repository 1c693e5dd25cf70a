// burgers2d -- 2D Burgers driver with the command line of the reference's 2D Burgers program
// (MultiGPU/Burgers2d_Baseline/main.c:38-49), on one GPU:
//   burgers2d tEnd CFL L W NX NY [block_x block_y] [--flags]
// Defaults follow that program's scheme: node grid dx = L/(N-1), local Lax-Friedrichs, WENO5-JS,
// inviscid, fixed dt = CFL dx (main.c:186), SSP-RK3, FP64, its Gaussian IC 3 (centred, zero on
// the outer ring; Tools.c:108-119). Boundary: three frozen layers (the 3D program's treatment),
// not that program's one-sided sweep ends. The grid is an nx x ny x 1 problem of the 3D solver.
// Flags:
//   --weno=z|js --lf=local|global --bc=frozen|periodic --viscosity=C --dt=fixed|maxu
//   --precision=f64|f32 --div=f32|f64 --max-steps=N --write=0|1 --out=result.bin
//   --checkpoint=state.bin --restart=state.bin
// With --bc=periodic the grid is cell-centred, dx = L/N.
#include <cmath>
#include <vector>

#include "driver_common.h"

int main(int argc, char** argv) {
  drv::Args a = drv::parse(argc, argv);
  if (a.pos.size() != 6 && a.pos.size() != 8) {
    std::printf("Usage: %s tEnd CFL L W NX NY [block_x block_y] [--weno=z|js] [--lf=local|global] "
                "[--bc=frozen|periodic] [--viscosity=C] [--dt=fixed|maxu] [--precision=f64|f32] [--div=f32|f64] "
                "[--max-steps=N] [--write=0|1] [--out=path] [--checkpoint=path] [--restart=path]\n", argv[0]);
    return 1;
  }
  const double tEnd = std::atof(a.pos[0].c_str()), CFL = std::atof(a.pos[1].c_str());
  const double L = std::atof(a.pos[2].c_str()), W = std::atof(a.pos[3].c_str());
  const int nx = std::atoi(a.pos[4].c_str()), ny = std::atoi(a.pos[5].c_str());
  const bool periodic = a.get("bc", "frozen") == "periodic";
  const double C = a.num("viscosity", 0.0);
  const int dtype = a.get("precision", "f64") == "f32" ? ADV_F32 : ADV_F64;
  adv_burgers_desc d{};
  d.nx = nx; d.ny = ny; d.nz = 1; d.dtype = dtype;
  d.weno = a.get("weno", "js") == "z" ? ADV_WENO5_Z : ADV_WENO5_JS;
  d.lf = a.get("lf", "local") == "global" ? ADV_LF_GLOBAL : ADV_LF_LOCAL;
  d.bc = periodic ? ADV_BC_PERIODIC : ADV_BC_FROZEN;
  d.div = a.get("div", "f32") == "f64" ? ADV_DIV_F64 : ADV_DIV_F32;
  d.dx = periodic ? L / nx : L / (nx - 1);
  d.dy = periodic ? W / ny : W / (ny - 1);
  d.dz = d.dx;  // unused: one plane
  d.kx = C / (12 * d.dx * d.dx); d.ky = C / (12 * d.dy * d.dy); d.kz = 0.0;
  const int rule = a.get("dt", "fixed") == "maxu" ? ADV_DT_MAXU : ADV_DT_FIXED;
  std::printf("dx: %g, dy: %g, final time: %g\n\n", d.dx, d.dy, tEnd);

  const size_t n = (size_t)nx * ny;
  std::vector<double> h(n);
  drv::check(adv_ic_burgers_ref2d(nx, ny, d.dx, d.dy, h.data()), "ic");
  const size_t es = dtype == ADV_F32 ? 4 : 8;
  std::vector<float> hf;
  const void* hsrc = h.data();
  if (dtype == ADV_F32) { hf.assign(h.begin(), h.end()); hsrc = hf.data(); }
  int64_t step0 = 0;
  double t0 = 0.0;
  drv::restart(a, dtype, nx, ny, 1, const_cast<void*>(hsrc), n * es, &step0, &t0, 0.0);

  cudaStream_t s;
  drv::check(cudaStreamCreate(&s), "stream");
  size_t wsb = 0;
  drv::check(adv_burgers_workspace_bytes(&d, &wsb), "workspace");
  void *du = nullptr, *dw = nullptr;
  drv::check(cudaMalloc(&du, n * es), "malloc");
  drv::check(cudaMalloc(&dw, wsb), "malloc");
  drv::Timer tm;
  tm.start(s);
  drv::check(cudaMemcpyAsync(du, hsrc, n * es, cudaMemcpyHostToDevice, s), "H2D");
  const double h2d = tm.stop(s);
  double t = 0;
  int64_t steps = 0;
  tm.start(s);
  drv::check(adv_burgers_resume(&d, du, dw, t0, step0, tEnd, CFL, rule, C, (int64_t)a.num("max-steps", 1e9), &t, &steps, s),
             "burgers run");
  const double secs = tm.stop(s);
  std::printf("Computation took %1.6f seconds\n\n", secs);
  std::printf("iterations: %lld, final time: %g\n\n", (long long)steps, t);
  tm.start(s);
  void* hdst = dtype == ADV_F32 ? (void*)hf.data() : (void*)h.data();
  drv::check(cudaMemcpyAsync(hdst, du, n * es, cudaMemcpyDeviceToHost, s), "D2H");
  const double d2h = tm.stop(s);
  drv::save_checkpoint(a, dtype, nx, ny, 1, steps, t, hdst);
  if (a.num("write", 0) != 0)
    drv::check(adv_write_result_bin(a.get("out", "result.bin").c_str(), dtype, hdst, (int64_t)n), "write");
  char grid[128], it[64];
  std::snprintf(grid, sizeof grid, "2D Grid Size                                 :  %d x %d", nx, ny);
  std::snprintf(it, sizeof it, "%lld x 3 RK steps", (long long)steps);
  drv::print_summary("Burgers-2D GPU-WENO5", "gb300 fused stage", secs, h2d, d2h,
                     (double)n * (steps - step0) * 3 / secs * 1e-9, grid, it, -1);
  cudaFree(du);
  cudaFree(dw);
  cudaStreamDestroy(s);
  return 0;
}
