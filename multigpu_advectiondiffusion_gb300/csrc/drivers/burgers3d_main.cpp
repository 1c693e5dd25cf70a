// burgers3d -- 3D Burgers driver with the reference's command line
// (SingleGPU/Burgers3d_WENO5/main.cpp:32-50; the 9-argument form of the SharedMem/Texture
// variants is accepted too):
//   burgers3d tEnd CFL L W H NX NY NZ [block_x block_y block_z] [--flags]
// Defaults reproduce the reference scheme: node grid dx = L/(N-1), local Lax-Friedrichs,
// WENO5-Z, viscous O4 term with C = 1e-5, three frozen layers, fixed dt = min(CFL dx,
// 0.9/(2C sum 1/h^2)), SSP-RK3, FP64, Gaussian IC 3. Flags:
//   --weno=z|js --lf=local|global --bc=frozen|periodic --viscosity=C --dt=fixed|maxu
//   --precision=f64|f32 --div=f32|f64 --ic=ref|fourier --seed=N --modes=16 --amax=0.1
//   --bug-b2=0|1 --max-steps=N --write=0|1 --out=result.bin
//   --checkpoint=state.bin (save the final state, step and t) --restart=state.bin (continue a
//   saved run to tEnd; a run stopped with --max-steps and continued takes the same steps, bit
//   for bit, as the uninterrupted run)
// With --bc=periodic the grid is cell-centred, dx = L/N.
#include <cmath>
#include <vector>

#include "driver_common.h"

int main(int argc, char** argv) {
  drv::Args a = drv::parse(argc, argv);
  if (a.pos.size() != 8 && a.pos.size() != 11) {
    std::printf("Usage: %s tEnd CFL L W H NX NY NZ [block_x block_y block_z] [--weno=z|js] [--lf=local|global] "
                "[--bc=frozen|periodic] [--viscosity=C] [--dt=fixed|maxu] [--precision=f64|f32] [--div=f32|f64] "
                "[--ic=ref|fourier] [--seed=N] [--bug-b2=0|1] [--max-steps=N] [--write=0|1] [--out=path] "
                "[--checkpoint=path] [--restart=path]\n", argv[0]);
    return 1;
  }
  const double tEnd = std::atof(a.pos[0].c_str()), CFL = std::atof(a.pos[1].c_str());
  const double L = std::atof(a.pos[2].c_str()), W = std::atof(a.pos[3].c_str()), H = std::atof(a.pos[4].c_str());
  const int nx = std::atoi(a.pos[5].c_str()), ny = std::atoi(a.pos[6].c_str()), nz = std::atoi(a.pos[7].c_str());
  const bool periodic = a.get("bc", "frozen") == "periodic";
  const double C = a.num("viscosity", periodic ? 0.0 : 1e-5);
  const int dtype = a.get("precision", "f64") == "f32" ? ADV_F32 : ADV_F64;
  adv_burgers_desc d{};
  d.nx = nx; d.ny = ny; d.nz = nz; d.dtype = dtype;
  d.weno = a.get("weno", "z") == "js" ? ADV_WENO5_JS : ADV_WENO5_Z;
  d.lf = a.get("lf", "local") == "global" ? ADV_LF_GLOBAL : ADV_LF_LOCAL;
  d.bc = periodic ? ADV_BC_PERIODIC : ADV_BC_FROZEN;
  d.div = a.get("div", "f32") == "f64" ? ADV_DIV_F64 : ADV_DIV_F32;
  d.bug_b2 = (int)a.num("bug-b2", 0);
  d.dx = periodic ? L / nx : L / (nx - 1);
  d.dy = periodic ? W / ny : W / (ny - 1);
  d.dz = periodic ? H / nz : H / (nz - 1);
  d.kx = C / (12 * d.dx * d.dx); d.ky = C / (12 * d.dy * d.dy); d.kz = C / (12 * d.dz * d.dz);
  const int rule = a.get("dt", "fixed") == "maxu" ? ADV_DT_MAXU : ADV_DT_FIXED;
  std::printf("dx: %g, dy: %g, dz: %g, final time: %g\n\n", d.dx, d.dy, d.dz, tEnd);

  const size_t n = (size_t)nx * ny * nz;
  std::vector<double> h(n);
  if (a.get("ic", "ref") == "fourier")
    drv::check(adv_ic_burgers_fourier(nx, ny, nz, L, (uint32_t)a.num("seed", 3), (int)a.num("modes", 16), a.num("amax", 0.1), h.data()), "ic");
  else
    drv::check(adv_ic_burgers_ref(nx, ny, nz, d.dx, d.dy, d.dz, h.data()), "ic");
  const size_t es = dtype == ADV_F32 ? 4 : 8;
  std::vector<float> hf;
  const void* hsrc = h.data();
  if (dtype == ADV_F32) { hf.assign(h.begin(), h.end()); hsrc = hf.data(); }
  int64_t step0 = 0;
  double t0 = 0.0;
  drv::restart(a, dtype, nx, ny, nz, const_cast<void*>(hsrc), n * (dtype == ADV_F32 ? 4 : 8), &step0, &t0, 0.0);

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
  drv::check(cudaMemcpyAsync(dtype == ADV_F32 ? (void*)hf.data() : (void*)h.data(), du, n * es, cudaMemcpyDeviceToHost, s), "D2H");
  const double d2h = tm.stop(s);
  drv::save_checkpoint(a, dtype, nx, ny, nz, steps, t, dtype == ADV_F32 ? (const void*)hf.data() : (const void*)h.data());
  if (a.num("write", 0) != 0)
    drv::check(adv_write_result_bin(a.get("out", "result.bin").c_str(), dtype,
                                    dtype == ADV_F32 ? (const void*)hf.data() : (const void*)h.data(), (int64_t)n), "write");
  char grid[128], it[64];
  std::snprintf(grid, sizeof grid, "3D Grid Size                                 :  %d x %d x %d", nx, ny, nz);
  std::snprintf(it, sizeof it, "%lld x 3 RK steps", (long long)steps);
  drv::print_summary("Burgers-3D GPU-WENO5", "gb300 fused stage", secs, h2d, d2h,
                     (double)n * (steps - step0) * 3 / secs * 1e-9,
                     grid, it, -1);
  cudaFree(du);
  cudaFree(dw);
  cudaStreamDestroy(s);
  return 0;
}
