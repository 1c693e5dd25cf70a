"""Benchmark: Gcell-updates/s per RK stage of the GB300 solvers.

Default workload (the configuration the metric is quoted on): 3D heat equation on a 256^3 node
grid, FP32, 7-point Laplacian, forward Euler with r = k dt/h^2 = 1/8, Dirichlet u = 0, initial
condition the sum of 8 seeded Gaussian blobs; one benchmark step = one full 2000-time-step solve.
Other workloads: --workload burgers3d (256^3 periodic WENO5-Z, global Lax-Friedrichs, SSP-RK3,
CFL 0.4; one benchmark step = 20 time steps).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload ...]

One JSON line on rank 0. `value` is device time with the state resident in HBM; `e2e` is the same
metric through the C ABI with the initial state copied from pinned host memory and the result
copied back inside the timed region. --impl reference times the reference scheme's CPU
restatement (the oracle) on all host cores for the same workload and metric.
Under torchrun each rank runs an independent replica (the path is single-GPU; no collective on
the data path) and value = total cell updates of all ranks / max rank time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

L2_BYTES = 126 * 1024 * 1024


def _peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def _traffic(workload: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary, or None."""
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get(workload)
        except Exception:
            return None
    return None


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while the timed region runs."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid: str | None):
        self.proc = None
        self.uuid = uuid

    def __enter__(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        if self.uuid:
            cmd += ["-i", self.uuid]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        time.sleep(0.25)
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, busy_mhz_floor: float = 0.0):
        rows = []
        for line in (self.out or "").splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) != 7:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), float(parts[2]), parts[3:]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower() == "active"})
        load = [r for r in rows if r[2] > 200.0] or rows
        sm = sorted(r[0] for r in load)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(r[2] for r in rows)}


# ----------------------------------------------------------------------------- workloads
def heat_setup(dtype):
    from oracle import oracle
    from multigpu_advectiondiffusion_gb300.solvers import HeatConfig
    n = 256
    cfg = HeatConfig.dirichlet_o2(3, n)
    u0 = oracle.ic_heat3d_blobs(n, n, n, 2).astype(dtype)
    return cfg, u0, 2000


def cpu_heat_rate(cfg, u0, budget_s: float):
    """Oracle (the reference scheme's CPU restatement) on all host threads: Gcell-updates/s."""
    from oracle import oracle
    t0 = time.perf_counter()
    oracle.heat_run(cfg, u0, 2, 0)
    one = (time.perf_counter() - t0) / 2
    steps = int(max(2, min(2000, budget_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    oracle.heat_run(cfg, u0, steps, 0)
    dt = time.perf_counter() - t0
    return cfg.numel * steps / dt / 1e9, steps, dt


def run_reference_arm(args, world, rank):
    from oracle import oracle
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    if args.workload == "heat3d":
        cfg, u0, nsteps = heat_setup(np.float32)
        per_step_budget = 2.0
        for _ in range(args.warmup):
            cpu_heat_rate(cfg, u0, 0.2)
        rates, samples = [], []
        t_all = 0.0
        for _ in range(args.steps):
            r, s, dt = cpu_heat_rate(cfg, u0, per_step_budget)
            rates.append(r)
            samples.append(s)
            t_all += dt
        value = float(np.median(rates))
        sample = f"256^3 FP32 O2 Euler, {int(np.median(samples))} of the 2000 time steps per step"
        config = {"workload": "heat3d 256^3 f32 o2 euler r=1/8 dirichlet 8 blobs x 2000 steps"}
    else:
        from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig
        n = 256
        cfg = BurgersConfig.periodic(n, weno="z")
        u0 = oracle.ic_burgers_fourier(n, n, n, 2.0, 3).astype(np.float32)
        rates = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            _, _, it = oracle.burgers_run(cfg, u0, 10.0, 0.4, 1, max_steps=1, div64=False)
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                rates.append(cfg.numel * 3 * it / dt / 1e9)
        value = float(np.median(rates))
        sample = "256^3 FP32 WENO5-Z periodic, 1 SSP-RK3 time step per step"
        config = {"workload": "burgers3d 256^3 f32 weno5-z global-lf periodic cfl 0.4"}
    line = {"impl": "reference", "metric": "Gcell-updates/s/RK-stage", "value": value, "unit": "Gcell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": config,
            "cpu_baseline": {"value": value, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="heat3d", choices=["heat3d", "burgers3d"])
    ap.add_argument("--cpu-budget", type=float, default=10.0, help="seconds of CPU-baseline work")
    ap.add_argument("--div", default="fast", choices=["fast", "f32", "f64"],
                    help="Burgers WENO weight division (FP32 state)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return

    import torch
    import torch.distributed as dist
    from multigpu_advectiondiffusion_gb300 import _native as N
    from multigpu_advectiondiffusion_gb300.solvers import (BurgersConfig, burgers_run, burgers_workspace, heat_run,
                                                           heat_workspace)

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            dist.barrier()

    lib = N.load()
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    if args.workload == "heat3d":
        cfg, u0_np, inner = heat_setup(np.float32)
        u0 = torch.from_numpy(u0_np).to(dev)
        u = u0.clone()
        ws = heat_workspace(cfg, u)
        launches_per_step = inner
        bytes_per_launch = 8 * cfg.numel
        cells_stages_per_step = cfg.numel * inner

        def one_step(uu):
            heat_run(cfg, uu, inner, ws, stream=sh)
        workload_name = "heat3d 256^3 f32 o2 euler r=1/8 dirichlet 8 blobs x 2000 steps"
        kernel = "heat_stage_kernel<float,2,3,TMA>"
    else:
        from oracle import oracle
        n = 256
        cfg = BurgersConfig.periodic(n, weno="z", div=args.div)
        u0 = torch.from_numpy(oracle.ic_burgers_fourier(n, n, n, 2.0, 3).astype(np.float32)).to(dev)
        u = u0.clone()
        ws = burgers_workspace(cfg, u)
        inner = 20
        launches_per_step = inner * 3  # stage kernels; the per-step dt kernels are timed with them
        bytes_per_launch = (8 + 12 + 12) / 3 * cfg.numel
        cells_stages_per_step = cfg.numel * 3 * inner

        def one_step(uu):
            burgers_run(cfg, uu, 1e9, 0.4, N.ADV_DT_MAXU, max_steps=inner, workspace=ws, stream=sh)
        workload_name = f"burgers3d 256^3 f32 weno5-z global-lf periodic cfl 0.4 x 20 steps, div {args.div}"
        kernel = f"burgers_stage_kernel<float,Z,{args.div}>"

    def timed(fn, K):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(K):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return ev0.elapsed_time(ev1)

    # ---- device-resident value
    for _ in range(args.warmup):
        one_step(u)
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    with ClockSampler(uuid) as clk:
        one_step(u)  # bring the clocks back up after the sampler's start-up pause
        launches0 = lib.adv_kernel_launch_count()
        ms = timed(lambda: one_step(u), args.steps)
        launched = lib.adv_kernel_launch_count() - launches0
    # time of the L2 flushes alone, subtracted from the per-launch figure only
    fl = timed(lambda: None, args.steps)
    ms_max = ms
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = t.item()
    value = world * cells_stages_per_step * args.steps / (ms_max * 1e-3) / 1e9
    launch_ms = (ms - fl) / max(1, args.steps * launches_per_step)
    achieved = bytes_per_launch / (launch_ms * 1e-3) / 1e9
    peak, peak_kind = _peaks()

    # ---- end to end through the C ABI from pinned host memory
    host_in = u0.cpu().pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()

    def e2e_step():
        with torch.cuda.stream(stream):
            u.copy_(host_in, non_blocking=True)
        one_step(u)
        with torch.cuda.stream(stream):
            host_out.copy_(u, non_blocking=True)
    for _ in range(2):
        e2e_step()
    ems = timed(e2e_step, args.steps)
    if world > 1:
        t = torch.tensor([ems], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ems = t.item()
    e2e_value = world * cells_stages_per_step * args.steps / (ems * 1e-3) / 1e9
    nbytes = u.numel() * u.element_size()

    # ---- accuracy of the FP32 result against FP64 (same device kernels, bit-exact with the oracle)
    extra = {}
    if args.workload == "heat3d":
        u32 = u0.clone()
        u64 = u0.double()
        heat_run(cfg, u32, inner, stream=sh)
        heat_run(cfg, u64, inner, stream=sh)
        torch.cuda.synchronize()
        extra["rel_l2_vs_fp64"] = (torch.linalg.vector_norm(u32.double() - u64) / torch.linalg.vector_norm(u64)).item()
        ws64 = heat_workspace(cfg, u64)
        for _ in range(2):
            heat_run(cfg, u64, inner, ws64, stream=sh)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(3):
            heat_run(cfg, u64, inner, ws64, stream=sh)
        ev1.record(stream)
        torch.cuda.synchronize()
        extra["f64_value"] = cells_stages_per_step * 3 / (ev0.elapsed_time(ev1) * 1e-3) / 1e9

    # ---- CPU baseline (oracle on the host cores, rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1 and args.workload == "heat3d":
        from oracle import oracle
        threads = os.cpu_count() or 1
        oracle.set_threads(threads)
        r, s, dtc = cpu_heat_rate(cfg, u0_np, args.cpu_budget)
        cpu = {"value": r, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
               "sample": f"256^3 FP32 O2 Euler, {s} time steps in {dtc:.1f} s (oracle, OpenMP)"}

    if rank == 0:
        line = {
            "metric": "Gcell-updates/s/RK-stage", "value": value, "unit": "Gcell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Philox4x32-10 initial condition)",
            "config": {"workload": workload_name, "parallelism": f"replicas{world}",
                       "l2": "per launch 64 MiB read + 64 MiB written > 126 MiB L2; 252 MiB L2 flush between steps"},
            "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "traffic": _traffic(args.workload),
                         "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_us": launch_ms * 1e3},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "Gcell-updates/s", "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes},
            "gpu_launches": int(launched),
            "clocks": clk.summary(),
            **extra,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
