// heat3d -- 3D heat-equation driver with the reference's command line
// (SingleGPU/Diffusion3d_baselineCode/main.cpp:32-50):
//   heat3d diffCoef L W H NX NY NZ n_iter [block_x block_y block_z] [--flags]
// Defaults reproduce the reference scheme: O4 13-point Laplacian, SSP-RK3 with
// dt = 0.9/(2C sum 1/h^2), two frozen boundary layers, FP64, the Gaussian IC 3 with t0 = 0.1,
// float32 result.bin. Flags select the other schemes:
//   --stencil=o2|o4  --time=euler|ssprk3  --bc=frozen|dirichlet  --precision=f64|f32
//   --ic=ref|blobs --seed=N --blobs=8  --r=<k dt/h^2 for Euler>  --write=0|1 --out=result.bin
//   --checkpoint=state.bin (save the final state, step count and time) --restart=state.bin
//   (continue a saved run: n_iter counts the whole run, so only the remaining steps are taken)
// L, W, H are integers as in the reference (atoi) unless --real-lengths is given.
#include <cmath>
#include <vector>

#include "driver_common.h"

int main(int argc, char** argv) {
  drv::Args a = drv::parse(argc, argv);
  if (a.pos.size() != 8 && a.pos.size() != 11) {
    std::printf("Usage: %s diffCoef L W H NX NY NZ n_iter [block_x block_y block_z] [--stencil=o2|o4] "
                "[--time=euler|ssprk3] [--bc=frozen|dirichlet] [--precision=f64|f32] [--ic=ref|blobs] [--seed=N] "
                "[--r=R] [--write=0|1] [--out=path] [--checkpoint=path] [--restart=path]\n", argv[0]);
    return 1;
  }
  const double C = std::atof(a.pos[0].c_str());
  const bool real_len = a.kv.count("real-lengths") > 0;
  const double L = real_len ? std::atof(a.pos[1].c_str()) : std::atoi(a.pos[1].c_str());
  const double W = real_len ? std::atof(a.pos[2].c_str()) : std::atoi(a.pos[2].c_str());
  const double H = real_len ? std::atof(a.pos[3].c_str()) : std::atoi(a.pos[3].c_str());
  const int nx = std::atoi(a.pos[4].c_str()), ny = std::atoi(a.pos[5].c_str()), nz = std::atoi(a.pos[6].c_str());
  const long iters = std::atol(a.pos[7].c_str());
  const int order = a.get("stencil", "o4") == "o2" ? 2 : 4;
  const int time = a.get("time", "ssprk3") == "euler" ? ADV_EULER : ADV_SSPRK3;
  const bool dirichlet = a.get("bc", "frozen") == "dirichlet";
  const int dtype = a.get("precision", "f64") == "f32" ? ADV_F32 : ADV_F64;
  const bool blobs = a.get("ic", "ref") == "blobs";

  const double dx = L / (nx - 1), dy = W / (ny - 1), dz = H / (nz - 1);
  double dt = 1 / (2 * C * (1 / dx / dx + 1 / dy / dy + 1 / dz / dz)) * 0.9;  // main.cpp:58
  if (a.kv.count("r")) dt = a.num("r", 0.125) * dx * dx / C;
  const double t0 = 0.1, tFinal = t0 + dt * iters;
  adv_heat_desc d{};
  d.ndim = 3; d.nx = nx; d.ny = ny; d.nz = nz; d.dtype = dtype; d.order = order;
  d.frozen = dirichlet ? order / 2 : 2;
  d.zero_boundary = dirichlet ? 1 : 0;
  if (order == 4) { d.kx = C / (12 * dx * dx); d.ky = C / (12 * dy * dy); d.kz = C / (12 * dz * dz); }
  else { d.kx = C / (dx * dx); d.ky = C / (dy * dy); d.kz = C / (dz * dz); }
  d.dt = dt;
  std::printf("dx: %g, dy: %g, dz: %g, dt: %g, final time: %g\n\n", dx, dy, dz, dt, tFinal);

  const size_t n = (size_t)nx * ny * nz;
  std::vector<double> h(n);
  if (blobs) drv::check(adv_ic_heat3d_blobs(nx, ny, nz, (uint32_t)a.num("seed", 2), (int)a.num("blobs", 8), h.data()), "ic");
  else drv::check(adv_ic_heat_ref(3, nx, ny, nz, dx, dy, dz, h.data()), "ic");
  const size_t es = dtype == ADV_F32 ? 4 : 8;
  std::vector<float> hf;
  const void* hsrc = h.data();
  if (dtype == ADV_F32) { hf.assign(h.begin(), h.end()); hsrc = hf.data(); }
  int64_t step0 = 0;
  double tstart = t0;
  drv::restart(a, dtype, nx, ny, nz, const_cast<void*>(hsrc), n * (dtype == ADV_F32 ? 4 : 8), &step0, &tstart, t0);
  const long todo = iters > step0 ? iters - (long)step0 : 0;

  cudaStream_t s;
  drv::check(cudaStreamCreate(&s), "stream");
  size_t wsb = 0;
  drv::check(adv_heat_workspace_bytes(&d, time, &wsb), "workspace");
  void *du = nullptr, *dw = nullptr;
  drv::check(cudaMalloc(&du, n * es), "malloc");
  drv::check(cudaMalloc(&dw, wsb), "malloc");
  drv::Timer tm;
  tm.start(s);
  drv::check(cudaMemcpyAsync(du, hsrc, n * es, cudaMemcpyHostToDevice, s), "H2D");
  const double h2d = tm.stop(s);
  tm.start(s);
  drv::check(adv_heat_run(&d, time, todo, du, dw, s), "heat run");
  const double secs = tm.stop(s);
  std::printf("Computation took %lf seconds\n", secs);
  tm.start(s);
  drv::check(cudaMemcpyAsync(dtype == ADV_F32 ? (void*)hf.data() : (void*)h.data(), du, n * es, cudaMemcpyDeviceToHost, s), "D2H");
  const double d2h = tm.stop(s);
  drv::save_checkpoint(a, dtype, nx, ny, nz, step0 + todo, t0 + dt * (double)(step0 + todo),
                       dtype == ADV_F32 ? (const void*)hf.data() : (const void*)h.data());
  const int stages = time == ADV_SSPRK3 ? 3 : 1;
  char grid[128], it[64];
  std::snprintf(grid, sizeof grid, "3D Grid Size                                 :  %d x %d x %d ", nx, ny, nz);
  std::snprintf(it, sizeof it, "%ld", iters);
  drv::print_summary(order == 4 ? "HeatEq3D (13-pt)" : "HeatEq3D (7-pt)", "gb300 fused stage", secs, h2d, d2h,
                     (double)n * todo * stages / secs * 1e-9, grid, it, tFinal);
  if (a.num("write", 1) != 0)
    drv::check(adv_write_result_bin(a.get("out", "result.bin").c_str(), dtype,
                                    dtype == ADV_F32 ? (const void*)hf.data() : (const void*)h.data(), (int64_t)n), "write");
  cudaFree(du);
  cudaFree(dw);
  cudaStreamDestroy(s);
  return 0;
}
