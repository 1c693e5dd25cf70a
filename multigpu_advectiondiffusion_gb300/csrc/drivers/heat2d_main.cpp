// heat2d -- 2D heat-equation driver with the reference's command line
// (SingleGPU/Diffusion2d/main.cpp:32-45):
//   heat2d diffCoef L W NX NY n_iter [block_x block_y] [--flags]
// Defaults reproduce the reference scheme: O4 9-point Laplacian, SSP-RK3 with
// dt = 0.9/(2C sum 1/h^2), three frozen boundary layers, FP64, Gaussian IC 3 with t0 = 0.1,
// float32 result.bin. Flags: --stencil=o2|o4 --time=euler|ssprk3 --bc=frozen|dirichlet
//   --precision=f64|f32 --ic=ref|gauss-noise --seed=N --sigma=1e-3 --r=R --write=0|1 --out=path
// L and W are integers as in the reference (atoi) unless --real-lengths is given.
#include <cmath>
#include <vector>

#include "driver_common.h"

int main(int argc, char** argv) {
  drv::Args a = drv::parse(argc, argv);
  if (a.pos.size() != 6 && a.pos.size() != 8) {
    std::printf("Usage: %s diffCoef L W NX NY n_iter [block_x block_y] [--stencil=o2|o4] [--time=euler|ssprk3] "
                "[--bc=frozen|dirichlet] [--precision=f64|f32] [--ic=ref|gauss-noise] [--seed=N] [--r=R] "
                "[--write=0|1] [--out=path]\n", argv[0]);
    return 1;
  }
  const double C = std::atof(a.pos[0].c_str());
  const bool real_len = a.kv.count("real-lengths") > 0;
  const double L = real_len ? std::atof(a.pos[1].c_str()) : std::atoi(a.pos[1].c_str());
  const double W = real_len ? std::atof(a.pos[2].c_str()) : std::atoi(a.pos[2].c_str());
  const int nx = std::atoi(a.pos[3].c_str()), ny = std::atoi(a.pos[4].c_str());
  const long iters = std::atol(a.pos[5].c_str());
  const int order = a.get("stencil", "o4") == "o2" ? 2 : 4;
  const int time = a.get("time", "ssprk3") == "euler" ? ADV_EULER : ADV_SSPRK3;
  const bool dirichlet = a.get("bc", "frozen") == "dirichlet";
  const int dtype = a.get("precision", "f64") == "f32" ? ADV_F32 : ADV_F64;
  const bool noise = a.get("ic", "ref") == "gauss-noise";

  const double dx = L / (nx - 1), dy = W / (ny - 1);
  double dt = 1 / (2 * C * (1 / dx / dx + 1 / dy / dy)) * 0.9;  // main.cpp:54
  if (a.kv.count("r")) dt = a.num("r", 0.2) * dx * dx / C;
  const double t0 = 0.1, tFinal = t0 + dt * iters;
  adv_heat_desc d{};
  d.ndim = 2; d.nx = nx; d.ny = ny; d.nz = 1; d.dtype = dtype; d.order = order;
  d.frozen = dirichlet ? order / 2 : 3;
  d.zero_boundary = dirichlet ? 1 : 0;
  if (order == 4) { d.kx = C / (12 * dx * dx); d.ky = C / (12 * dy * dy); }
  else { d.kx = C / (dx * dx); d.ky = C / (dy * dy); }
  d.dt = dt;
  std::printf("dx: %g, dy: %g, dt: %g, final time: %g\n\n", dx, dy, dt, tFinal);

  const size_t n = (size_t)nx * ny;
  std::vector<double> h(n);
  if (noise) drv::check(adv_ic_heat2d_gauss_noise(nx, ny, (uint32_t)a.num("seed", 1), a.num("sigma", 1e-3), h.data()), "ic");
  else drv::check(adv_ic_heat_ref(2, nx, ny, 1, dx, dy, 0.0, h.data()), "ic");
  const size_t es = dtype == ADV_F32 ? 4 : 8;
  std::vector<float> hf;
  const void* hsrc = h.data();
  if (dtype == ADV_F32) { hf.assign(h.begin(), h.end()); hsrc = hf.data(); }

  cudaStream_t s;
  drv::check(cudaStreamCreate(&s), "stream");
  size_t wsb = 0;
  drv::check(adv_heat_workspace_bytes(&d, time, &wsb), "workspace");
  void *du = nullptr, *dw = nullptr;
  drv::check(cudaMalloc(&du, n * es), "malloc");
  drv::check(cudaMalloc(&dw, wsb), "malloc");
  drv::Timer tm;
  drv::check(cudaMemcpyAsync(du, hsrc, n * es, cudaMemcpyHostToDevice, s), "H2D");
  tm.start(s);
  drv::check(adv_heat_run(&d, time, iters, du, dw, s), "heat run");
  const double secs = tm.stop(s);
  std::printf("Computation took %lf seconds\n", secs);
  drv::check(cudaMemcpyAsync(dtype == ADV_F32 ? (void*)hf.data() : (void*)h.data(), du, n * es, cudaMemcpyDeviceToHost, s), "D2H");
  drv::check(cudaStreamSynchronize(s), "sync");
  const int stages = time == ADV_SSPRK3 ? 3 : 1;
  char grid[128], it[64];
  std::snprintf(grid, sizeof grid, "2D Grid Size                                 :  %d x %d ", nx, ny);
  std::snprintf(it, sizeof it, "%ld", iters);
  drv::print_summary(order == 4 ? "HeatEq2D (13-pt)" : "HeatEq2D (5-pt)", "gb300 fused stage", secs, -1, -1,
                     (double)n * iters * stages / secs * 1e-9, grid, it, tFinal);
  if (a.num("write", 1) != 0)
    drv::check(adv_write_result_bin(a.get("out", "result.bin").c_str(), dtype,
                                    dtype == ADV_F32 ? (const void*)hf.data() : (const void*)h.data(), (int64_t)n), "write");
  cudaFree(du);
  cudaFree(dw);
  cudaStreamDestroy(s);
  return 0;
}
