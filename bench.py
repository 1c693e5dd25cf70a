"""Benchmark: Gcell-updates/s per RK stage of the GB300 solvers.

Default workload (the configuration the metric is quoted on): 3D heat equation on a 256^3 node
grid, FP32, 7-point Laplacian, forward Euler with r = k dt/h^2 = 1/8, Dirichlet u = 0, initial
condition the sum of 8 seeded Gaussian blobs; one benchmark step = one full 2000-time-step solve.
Other workloads: --workload burgers3d (256^3 periodic WENO5-Z, global Lax-Friedrichs, SSP-RK3,
CFL 0.4; one benchmark step = 20 time steps); --workload ensemble (64 heat + 32 Burgers 3D
instances of uneven size advanced by one CUDA graph, 500 steps each; one benchmark step = one
ensemble run; also times the plain per-instance loop over the same instances).

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
import dataclasses
import ctypes as C
import json
import os
import platform
import re
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

L2_BYTES = 126 * 1024 * 1024


def settle(step, seconds: float = 2.0, max_steps: int = 1000) -> None:
    """Untimed steps until `seconds` of wall time have passed after the warm-up (clocks and
    caches in their steady state before the timed region)."""
    import torch
    t_end = time.perf_counter() + seconds
    for _ in range(max_steps):
        step()
        torch.cuda.synchronize()
        if time.perf_counter() >= t_end:
            break


def prime_device(local: int) -> None:
    """Creates and releases one CUDA context on this rank's GPU in a short-lived child process
    before this process creates its own. Measured on freshly started boxes: when the benchmark
    was the first process to use the GPU, its memory-bound kernels ran 35% slower for the whole
    process (heat 497 vs 771 Gcell/s; the same code, shapes and clocks, and every later process
    fast), and one earlier process that only created a context removed the difference."""
    code = f"import torch; torch.zeros(1, device='cuda:{local}'); torch.cuda.synchronize()"
    try:
        subprocess.run([sys.executable, "-c", code], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL,
                       timeout=300, check=False)
    except (OSError, subprocess.SubprocessError):
        pass


def max_over_ranks(x: float, device=None) -> float:
    """The largest of every rank's x (the job's time is its slowest replica's); x itself when the
    job has one rank or no process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, ms_max: float, world: int) -> float:
    """Whole-job throughput in G units/s: every rank processes units_per_rank in its replica, and
    the job takes as long as its slowest rank (ms_max)."""
    return world * units_per_rank / (ms_max * 1e-3) / 1e9


def _peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


TRAFFIC_NOTE = ("dram__bytes_read.sum + dram__bytes_write.sum of one ncu-captured launch (profiles/traffic.json); "
                "writes still dirty in L2 when that launch ends are not counted, so it can sit below the "
                "algorithmic bytes even though every node is written once per launch")


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
def ic_heat3d_blobs(nx, ny, nz, seed, nblobs=8, source="library"):
    """Seeded initial condition from the library's host generator (adv_ic_heat3d_blobs), or the
    oracle's (source="oracle", for the CPU arms: equal bit for bit)."""
    if source == "oracle":
        from oracle import oracle
        return oracle.ic_heat3d_blobs(nx, ny, nz, seed, nblobs)
    from multigpu_advectiondiffusion_gb300 import _native as N
    u = np.empty(nx * ny * nz)
    N.check(N.load().adv_ic_heat3d_blobs(nx, ny, nz, seed, nblobs, u.ctypes.data_as(C.POINTER(C.c_double))), "ic")
    return u


def ic_burgers_fourier(nx, ny, nz, L, seed, nmodes=16, amax=0.1, source="library"):
    """Seeded initial condition from the library's host generator (adv_ic_burgers_fourier), or the
    oracle's (source="oracle")."""
    if source == "oracle":
        from oracle import oracle
        return oracle.ic_burgers_fourier(nx, ny, nz, L, seed, nmodes, amax)
    from multigpu_advectiondiffusion_gb300 import _native as N
    u = np.empty(nx * ny * nz)
    N.check(N.load().adv_ic_burgers_fourier(nx, ny, nz, L, seed, nmodes, amax,
                                            u.ctypes.data_as(C.POINTER(C.c_double))), "ic")
    return u


HEAT3D_WORKLOAD = "heat3d 256^3 f32 o2 euler r=1/8 dirichlet 8 blobs x 2000 steps"
HEAT2D_WORKLOAD = "heat2d 512^2 f32 o2 euler r=0.2 dirichlet gaussian bump + N(0,1e-3) noise x 1000 steps"


def heat_case(workload: str):
    """(config, time steps per solve) of a heat workload: 3D 256^3 O2 forward Euler at r = 1/8 for
    2000 steps (the metric's configuration), or 2D 512^2 O2 forward Euler at r = 0.2 for 1000 steps
    (the plain method, CPU-sized). The configuration object is a plain dataclass (no library load)."""
    from multigpu_advectiondiffusion_gb300.solvers import HeatConfig
    if workload == "heat2d":
        return HeatConfig.dirichlet_o2(2, 512), 1000
    return HeatConfig.dirichlet_o2(3, 256), 2000


def heat_initial(workload: str, source: str = "library") -> np.ndarray:
    """The workload's seeded FP32 initial state, from the library's host generator (the GPU arm) or
    the oracle's (the CPU arms; the two are equal bit for bit, tests/test_abi.py)."""
    cfg, _ = heat_case(workload)
    if source == "oracle":
        from oracle import oracle
        u = (oracle.ic_heat2d_gauss_noise(cfg.nx, cfg.ny, 1, 1e-3) if workload == "heat2d"
             else oracle.ic_heat3d_blobs(cfg.nx, cfg.ny, cfg.nz, 2))
        return u.astype(np.float32)
    if workload == "heat2d":
        from multigpu_advectiondiffusion_gb300 import _native as N
        u = np.empty(cfg.nx * cfg.ny)
        N.check(N.load().adv_ic_heat2d_gauss_noise(cfg.nx, cfg.ny, 1, 1e-3, u.ctypes.data_as(C.POINTER(C.c_double))),
                "ic")
        return u.astype(np.float32)
    return ic_heat3d_blobs(cfg.nx, cfg.ny, cfg.nz, 2).astype(np.float32)


def heat_config(workload: str, world: int) -> dict:
    """The `config` object both arms print for a heat workload (identical, so the two lines can be
    matched)."""
    if workload == "heat2d":
        return {"workload": HEAT2D_WORKLOAD, "parallelism": f"replicas{world}",
                "l2": "1 MiB state fits in L2 (the plain method's size); 252 MiB L2 flush between GPU steps"}
    return {"workload": HEAT3D_WORKLOAD, "parallelism": f"replicas{world}",
            "l2": "per time step 64 MiB read + 64 MiB written > 126 MiB L2; 252 MiB L2 flush between GPU steps"}


def cpu_heat_rate(cfg, u0, nsteps: int, budget_s: float):
    """The tuned CPU loop (oracle/cpu_baseline.cpp: the same O2 forward-Euler update, OpenMP) on a
    bounded sample of one solve: min(nsteps, what fits in about budget_s) time steps from u0.
    Returns (Gcell-updates/s, time steps, seconds)."""
    from oracle import oracle
    u = u0.copy()
    w = np.empty_like(u)
    t0 = time.perf_counter()
    oracle.cpu_heat_euler_o2(cfg, u, 2, w)
    one = (time.perf_counter() - t0) / 2
    steps = int(max(2, min(nsteps, budget_s / max(one, 1e-9))))
    u[:] = u0
    t0 = time.perf_counter()
    oracle.cpu_heat_euler_o2(cfg, u, steps, w)
    dt = time.perf_counter() - t0
    return cfg.numel * steps / dt / 1e9, steps, dt


def cpu_model() -> str:
    """The host CPU's name: /proc/cpuinfo's model name (x86) or implementer/part codes (Arm)."""
    try:
        txt = Path("/proc/cpuinfo").read_text()
    except OSError:
        return platform.machine()
    m = re.search(r"^model name\s*:\s*(.+)$", txt, re.M)
    if m:
        return m.group(1).strip()
    part = re.search(r"^CPU part\s*:\s*(\S+)$", txt, re.M)
    impl = re.search(r"^CPU implementer\s*:\s*(\S+)$", txt, re.M)
    if part:
        known = {("0x41", "0xd4f"): "Arm Neoverse-V2"}
        key = (impl.group(1) if impl else "", part.group(1))
        return known.get(key, f"{platform.machine()} implementer {key[0]} part {key[1]}")
    return platform.machine()


def cpu_baseline_heat(cfg, u0, nsteps: int, budget_s: float) -> dict:
    """The tuned CPU loop's rate on the heat workload with all host threads, then on one thread
    (bounded samples of about budget_s and min(budget_s, 3) seconds)."""
    from oracle import oracle
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    r, s, dtc = cpu_heat_rate(cfg, u0, nsteps, budget_s)
    oracle.set_threads(1)
    try:
        r1, s1, dt1 = cpu_heat_rate(cfg, u0, nsteps, min(budget_s, 3.0))
    finally:
        oracle.set_threads(threads)
    size = f"{cfg.nx}^{cfg.ndim}"
    return {"value": r, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
            "sample": f"{size} FP32 O2 Euler, {s} of the {nsteps} time steps in {dtc:.2f} s (tuned CPU loop, "
                      "oracle/cpu_baseline.cpp, OpenMP)",
            "one_core_value": r1, "one_core_sample": f"{s1} time steps in {dt1:.2f} s on one thread",
            "cpu_model": cpu_model()}


# FP32 flops per cell-stage of the fused WENO5-Z stage, counting an FFMA2 as 4 flops, an FADD2,
# FMUL2 or FFMA as 2 and an FADD or FMUL as 1, from the ncu instruction mix of the
# reciprocal-division form at 256^3 (stage 1): FFMA2 81.2, FADD2 18.5, FMUL2 37.3, FFMA 6.6,
# FADD 5.3, FMUL 10.1 per cell = 465.0. The division counts as the reciprocal form's operations
# whichever division is run.
BURGERS_FLOPS_PER_CELL_STAGE = 465.0

ENSEMBLE_SEED = 2024
ENSEMBLE_STEPS = 500
# WENO weight division of the ensemble's Burgers members: in FP64 (its quotient rounded to the FP32
# state is also the IEEE FP32 division's, bit for bit: tests/test_gpu_burgers.py; the two measure
# the same speed)
ENSEMBLE_DIV = "f64"


def ensemble_workload() -> str:
    return (f"ensemble 64 heat (n in 64..192, o2 euler r=1/8) + 32 burgers (n in 96..160, weno5-z global-lf "
            f"periodic cfl 0.4, {DIV_LABEL[ENSEMBLE_DIV]} div) x {ENSEMBLE_STEPS} steps, one graph")


def ensemble_members():
    """The batched-ensemble workload: 64 heat instances, n^3 with n uniform in {64,96,128,160,192},
    diffusivity log-uniform in [0.1, 10], O2 forward Euler at r = 1/8 (dt per instance), Dirichlet
    u = 0, 8 seeded Gaussian blobs each; 32 periodic WENO5-Z global-LF Burgers instances, n^3 with n
    uniform in {96,112,128,144,160}, seeded 16-mode Fourier initial conditions, CFL 0.4. FP32."""
    from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig, HeatConfig
    rng = np.random.default_rng(ENSEMBLE_SEED)
    heat = []
    for _ in range(64):
        n = int(rng.choice([64, 96, 128, 160, 192]))
        k = float(10 ** rng.uniform(-1, 1))
        heat.append(HeatConfig.dirichlet_o2(3, n, k=k, r=0.125))
    burgers = [BurgersConfig.periodic(int(rng.choice([96, 112, 128, 144, 160])), weno="z", div=ENSEMBLE_DIV)
               for _ in range(32)]
    return heat, burgers


def ensemble_initial_states(heat, burgers, source="library"):
    hs = [ic_heat3d_blobs(c.nx, c.ny, c.nz, 100 + i, source=source).astype(np.float32) for i, c in enumerate(heat)]
    bs = [ic_burgers_fourier(c.nx, c.ny, c.nz, 2.0, 200 + i, source=source).astype(np.float32)
          for i, c in enumerate(burgers)]
    return hs, bs


def ensemble_config(world: int) -> dict:
    return {"workload": ensemble_workload(), "parallelism": f"replicas{world}",
            "l2": "1.5 GB heat + 0.9 GB Burgers state > 126 MiB L2; 252 MiB L2 flush between GPU steps"}


def bench_ensemble(args, world, rank, dev, stream, flush, lib):
    import torch
    import torch.distributed as dist
    from multigpu_advectiondiffusion_gb300 import _native as N
    from multigpu_advectiondiffusion_gb300.solvers import (Ensemble, burgers_run, burgers_workspace, heat_run,
                                                           heat_workspace)
    heat, burgers = ensemble_members()
    h0, b0 = ensemble_initial_states(heat, burgers)
    hu = [torch.from_numpy(a).to(dev) for a in h0]
    bu = [torch.from_numpy(a).to(dev) for a in b0]
    S = ENSEMBLE_STEPS
    ens = Ensemble(heat=list(zip(heat, hu)), burgers=[(c, u, 1e9, 0.4, N.ADV_DT_MAXU, S) for c, u in zip(burgers, bu)])
    sh = stream.cuda_stream
    heat_cells = sum(c.numel for c in heat)
    burg_cells = sum(c.numel for c in burgers)
    work = heat_cells * S + burg_cells * 3 * S  # cell updates per RK stage in one ensemble run

    def barrier():
        if world > 1:
            dist.barrier()

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

    def reset():
        for u, a in zip(hu + bu, h0 + b0):
            u.copy_(torch.from_numpy(a).to(dev), non_blocking=False)

    def one_step():
        ens.run(S, stream=sh)

    for _ in range(args.warmup):
        reset()
        one_step()
    settle(one_step)
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    # Each timed step starts from the same initial states (reset outside the timed region would
    # need K separate regions; the states stay bounded over repeated runs, so the runs continue).
    reset()
    with ClockSampler(uuid) as clk:
        settle(one_step, 1.0)  # the sampler's start-up (NVML) overlaps untimed work
        launches0 = lib.adv_kernel_launch_count()
        ms = timed(one_step, args.steps)
        launched = lib.adv_kernel_launch_count() - launches0
    ms_max = max_over_ranks(ms, dev)
    value = replica_throughput(work * args.steps, ms_max, world)

    # Burgers loop alone (heat_steps = 0): the batched WENO stage dominates; its average launch
    # time is this loop's time over its 3 S stage launches (the per-step dt kernel included).
    ms_b = timed(lambda: ens.run(0, stream=sh), 1)
    fl = timed(lambda: None, 1)
    launch_ms = (ms_b - fl) / (3 * S)
    bytes_per_launch = (8 + 12 + 12) / 3 * burg_cells
    achieved = bytes_per_launch / (launch_ms * 1e-3) / 1e9
    peak, peak_kind = _peaks()

    # heat members alone in their own ensemble: the batched heat stage is HBM-bound; one Euler
    # step is one launch over all 64 instances (8 B per node: read u, write u')
    ens_h = Ensemble(heat=list(zip(heat, hu)))
    ens_h.run(S, stream=sh)
    ms_h = timed(lambda: ens_h.run(S, stream=sh), 1)
    heat_launch_ms = (ms_h - fl) / S
    heat_bytes = 8 * heat_cells
    heat_achieved = heat_bytes / (heat_launch_ms * 1e-3) / 1e9
    heat_shape = ens_h.shape()
    ens_h.close()

    # launch floor: the same graph (64 heat + 32 Burgers members, S steps, the same per-step
    # kernels and stage launches) over 16^3 heat and 32^3 Burgers members, whose launches carry
    # almost no work. What this run costs bounds what fusing the loop into one persistent kernel
    # could remove (launch gaps, graph node overhead and the per-step kernels).
    from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig, HeatConfig
    gen = torch.Generator(device="cpu").manual_seed(ENSEMBLE_SEED)
    th = [HeatConfig.dirichlet_o2(3, 16, r=0.125) for _ in heat]
    tb = [BurgersConfig.periodic(32, weno="z", div=ENSEMBLE_DIV) for _ in burgers]
    thu = [torch.rand(c.numel, generator=gen).to(dev) for c in th]
    tbu = [(0.5 + 0.1 * torch.rand(c.numel, generator=gen)).to(dev) for c in tb]
    ens_t = Ensemble(heat=list(zip(th, thu)), burgers=[(c, u, 1e9, 0.4, N.ADV_DT_MAXU, S) for c, u in zip(tb, tbu)])
    ens_t.run(S, stream=sh)
    floor_ms = timed(lambda: ens_t.run(S, stream=sh), 1) - fl
    ens_t.close()

    # plain per-instance loop over the same instances (each instance its own heat_run /
    # burgers_run: one-wave grids per instance, one graph per instance)
    hws = [heat_workspace(c, u) for c, u in zip(heat, hu)]
    bws = [burgers_workspace(c, u) for c, u in zip(burgers, bu)]

    def loop_step():
        for c, u, w in zip(heat, hu, hws):
            heat_run(c, u, S, w, stream=sh)
        for c, u, w in zip(burgers, bu, bws):
            burgers_run(c, u, 1e9, 0.4, N.ADV_DT_MAXU, max_steps=S, workspace=w, stream=sh)
    loop_step()
    ms_loop = timed(loop_step, 1)
    loop_value = work / (ms_loop * 1e-3) / 1e9

    # end to end: every instance's state from pinned host memory, results back
    host_in = [torch.from_numpy(a).pin_memory() for a in h0 + b0]
    host_out = [torch.empty_like(a) .pin_memory() for a in host_in]
    dev_all = hu + bu

    def e2e_step():
        with torch.cuda.stream(stream):
            for d, h in zip(dev_all, host_in):
                d.copy_(h, non_blocking=True)
        one_step()
        with torch.cuda.stream(stream):
            for h, d in zip(host_out, dev_all):
                h.copy_(d, non_blocking=True)
    e2e_step()
    ems = max_over_ranks(timed(e2e_step, args.steps), dev)
    nbytes = sum(a.numel() * a.element_size() for a in host_in)
    shape = ens.shape()
    ens.close()
    if rank == 0:
        line = {
            "metric": "Gcell-updates/s/RK-stage", "value": value, "unit": "Gcell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded sizes, diffusivities and Philox4x32-10 initial conditions)",
            "config": ensemble_config(world),
            "shape": {"heat_cells": heat_cells, "burgers_cells": burg_cells, **shape},
            "roofline": {"bound": "hbm", "kernel": f"burgers_batch_kernel<float,Z,{ENSEMBLE_DIV} div>", "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": _traffic("ensemble"), "algorithmic_bytes_per_launch": bytes_per_launch,
                         "avg_launch_us": launch_ms * 1e3},
            "cpu_baseline": cpu_baseline_sample(args, world) if world == 1 else None,
            "e2e": {"value": replica_throughput(work * args.steps, ems, world), "unit": "Gcell-updates/s",
                    "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
            "gpu_launches": int(launched),
            "clocks": clk.summary(),
            "launch_floor": {"ms_per_run": floor_ms, "share_of_run": floor_ms / (ms_max / args.steps),
                             "measured_as": "the same graph over 64 heat 16^3 + 32 Burgers 32^3 members, "
                                            f"{S} steps: launches carrying almost no work"},
            "per_instance_loop_value": loop_value,
            "speedup_vs_per_instance_loop": value / loop_value,
            "roofline_heat_batch": {"bound": "hbm", "kernel": "heat_batch_kernel<float,2,TMA,stage 1>",
                                    "achieved": heat_achieved, "peak": peak, "unit": "GB/s",
                                    "frac": heat_achieved / peak, "peak_source": peak_kind,
                                    "algorithmic_bytes_per_launch": heat_bytes,
                                    "avg_launch_us": heat_launch_ms * 1e3,
                                    "heat_value": heat_cells / (heat_launch_ms * 1e-3) / 1e9,
                                    "measured_as": "the 64 heat instances alone in one ensemble, 500 Euler steps",
                                    **{k: v for k, v in heat_shape.items() if k.startswith("heat")}},
        }
        print(json.dumps(line), flush=True)


ADJ_N, ADJ_STEPS, ADJ_INTERVAL, ADJ_T = 128, 400, 20, 0.15
HEATK_N, HEATK_STEPS = 192, 200


def adjoint_setup():
    """Config of the discrete-adjoint workload: Burgers WENO5-Z, local LF, periodic [0,2)^3 at 128^3
    FP32, 400 SSP-RK3 steps of a fixed dt = 0.15 / 400 from the seeded Fourier state (seed 5), i.e.
    to t = 0.15, before the first shocks (past them the discrete adjoint of a captured shock is
    dominated by rounding-level sensitivities and no finite difference can check it);
    u_target = the forward result of seed 6; checkpoints every 20 steps. Heat: 192^3 FP32, k(x) =
    exp(g) with g a box-smoothed N(0, 0.25) field (seed 23), dt k_max / h^2 = 1/8, 200 steps, 8
    seeded blobs, target = the forward result of another diffusivity draw (seed 24)."""
    from multigpu_advectiondiffusion_gb300 import _native as N
    from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig, HeatKConfig
    n = ADJ_N
    bc = BurgersConfig(n, n, n, 2.0 / n, 2.0 / n, 2.0 / n, N.ADV_WENO5_Z, N.ADV_LF_LOCAL, N.ADV_BC_PERIODIC,
                       N.ADV_DIV_FAST)
    u0 = ic_burgers_fourier(n, n, n, 2.0, 5)
    ut = ic_burgers_fourier(n, n, n, 2.0, 6)
    dt = ADJ_T / ADJ_STEPS
    m = HEATK_N

    def kfield(seed):
        g = np.random.default_rng(seed).normal(0.0, 0.5, (m, m, m))
        for ax in range(3):
            g = (np.roll(g, 1, ax) + g + np.roll(g, -1, ax)) / 3.0
        return np.exp(g / g.std() * 0.5).ravel()

    k = kfield(23)
    k2 = kfield(24)
    hc = HeatKConfig.cube(m, 0.125, float(max(k.max(), k2.max())))
    h0 = ic_heat3d_blobs(m, m, m, 2)
    return bc, u0, ut, dt, hc, k, k2, h0


def bench_adjoint(args, world, rank, dev, lib):
    import torch
    from multigpu_advectiondiffusion_gb300.solvers import auto_interval, burgers_run_fixed, default_interval, heatk_run
    bc, u0n, utn, dt, hc, kn, k2n, h0n = adjoint_setup()
    u0 = torch.from_numpy(u0n.astype(np.float32)).to(dev)
    # checkpoint spacing the library's wrappers choose by default: the whole run kept when it fits
    # in half the free HBM (here: every stage input, no recompute), else sqrt(N)
    iv_b = auto_interval(ADJ_STEPS, 3, u0)
    with torch.no_grad():
        target = burgers_run_fixed(bc, torch.from_numpy(utn.astype(np.float32)).to(dev), dt, ADJ_STEPS, ADJ_INTERVAL)

    def ev(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        r = fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b), r

    def grad_burgers(u, tgt, interval=iv_b):
        uu = u.clone().requires_grad_(True)
        tf, uT = ev(lambda: burgers_run_fixed(bc, uu, dt, ADJ_STEPS, interval))
        loss = 0.5 * ((uT - tgt) ** 2).sum()
        tb, _ = ev(loss.backward)
        return tf, tb, uu.grad, float(loss.detach())

    for _ in range(args.warmup):
        grad_burgers(u0, target)
    settle(lambda: grad_burgers(u0, target))
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    tfs, tbs = [], []
    with ClockSampler(uuid) as clk:
        launches0 = lib.adv_kernel_launch_count()
        for _ in range(args.steps):
            tf, tb, g32, J32 = grad_burgers(u0, target)
            tfs.append(tf)
            tbs.append(tb)
        launched = lib.adv_kernel_launch_count() - launches0
    tf, tb = float(np.median(tfs)), float(np.median(tbs))
    cells = ADJ_N ** 3 * 3 * ADJ_STEPS
    # sqrt(N) checkpoints (every ADJ_INTERVAL steps): the backward run recomputes every interval
    sq = [grad_burgers(u0, target, ADJ_INTERVAL) for _ in range(3)]
    tf_s, tb_s = float(np.median([r[0] for r in sq])), float(np.median([r[1] for r in sq]))
    assert torch.equal(sq[0][2], g32), "the gradient depends on the checkpoint spacing"
    # FP64 adjoint and central differences of the FP64 forward along 16 seeded directions
    u64 = u0.double()
    t64 = target.double()
    _, _, g64, _ = grad_burgers(u64, t64, ADJ_INTERVAL)
    rel64 = (torch.linalg.vector_norm(g32.double() - g64) / torch.linalg.vector_norm(g64)).item()

    def J64(u):
        with torch.no_grad():
            return 0.5 * float(((burgers_run_fixed(bc, u, dt, ADJ_STEPS, ADJ_INTERVAL) - t64) ** 2).sum())

    fd_err = []
    for i in range(16):
        d = torch.from_numpy(np.random.default_rng(7 + i).standard_normal(u0.numel())).to(dev)
        eps = 1e-8
        fd = (J64(u64 + eps * d) - J64(u64 - eps * d)) / (2 * eps)
        ad = float((g32.double() * d).sum())
        fd_err.append(abs(fd - ad) / abs(fd))
    # heat with k(x): gradient w.r.t. k and u0
    k = torch.from_numpy(kn.astype(np.float32)).to(dev)
    h0 = torch.from_numpy(h0n.astype(np.float32)).to(dev)
    with torch.no_grad():
        htarget = heatk_run(hc, torch.from_numpy(k2n.astype(np.float32)).to(dev), h0, HEATK_STEPS)

    if not args.no_tune:
        from multigpu_advectiondiffusion_gb300.solvers import autotune_heatk
        autotune_heatk(hc, k, h0)

    def grad_heat(interval=None):
        kk = k.clone().requires_grad_(True)
        hh = h0.clone().requires_grad_(True)
        tfh, uT = ev(lambda: heatk_run(hc, kk, hh, HEATK_STEPS, interval))
        loss = 0.5 * ((uT - htarget) ** 2).sum()
        tbh, _ = ev(loss.backward)
        return tfh, tbh

    def median_grad(interval=None):
        for _ in range(2):
            grad_heat(interval)
        hts = [grad_heat(interval) for _ in range(3)]
        return float(np.median([h[0] for h in hts])), float(np.median([h[1] for h in hts]))
    iv_h = auto_interval(HEATK_STEPS, 1, h0)
    tfh, tbh = median_grad(iv_h)
    tfh_s, tbh_s = median_grad(default_interval(HEATK_STEPS))

    def kept(iv, nsteps, arrays, one_b=0):
        if iv >= nsteps:
            return (f"whole run kept ({arrays} arrays, {arrays * one_b / 1e9:.1f} GB of HBM; the default when it "
                    f"fits in half the free memory): no recompute")
        return f"every {iv} steps (sqrt N; the default when the whole run does not fit)"
    t_grad = max_over_ranks(tf + tb, dev)
    if rank == 0:
        line = {
            "metric": "Gcell-updates/s/RK-stage", "value": replica_throughput(cells, t_grad, world),
            "unit": "Gcell-updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_grad, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Fourier states and log-normal diffusivity)",
            "config": adjoint_config(world),
            "value_is": "forward cell-stage updates per second of forward + backward (one gradient)",
            "scheme_differentiated": (f"WENO5-Z, local Lax-Friedrichs, periodic, fixed dt (CFL "
                                      f"{dt * float(u0.abs().max()) / bc.dx:.3f} at t = 0), SSP-RK3; the C3 forward "
                                      "uses global LF, whose max|u| constant the adjoint does not differentiate"),
            "roofline": None,
            "cpu_baseline": cpu_baseline_sample(args, world) if world == 1 else None,
            "e2e": None,
            "gpu_launches": int(launched),
            "clocks": clk.summary(),
            "burgers": {"forward_ms": tf, "backward_ms": tb, "backward_over_forward": tb / tf,
                        "forward_value": cells / (tf * 1e-3) / 1e9, "grad_fp32_vs_fp64_rel_l2": rel64,
                        "fd_rel_err_max_16_dirs": max(fd_err), "fd_rel_err_median": float(np.median(fd_err)),
                        "fd": "central differences of the FP64 forward run, step 1e-8, 16 seeded directions",
                        "checkpoints": kept(iv_b, ADJ_STEPS, 3 * min(iv_b, ADJ_STEPS) + 3, ADJ_N ** 3 * 4)},
            "burgers_sqrt_n": {"forward_ms": tf_s, "backward_ms": tb_s, "backward_over_forward": tb_s / tf_s,
                               "checkpoints": kept(ADJ_INTERVAL, ADJ_STEPS, 0),
                               "gradient": "bit-identical to the kept run's"},
            "heat_k": {"forward_ms": tfh, "backward_ms": tbh, "backward_over_forward": tbh / tfh,
                       "forward_value": HEATK_N ** 3 * HEATK_STEPS / (tfh * 1e-3) / 1e9,
                       "checkpoints": kept(iv_h, HEATK_STEPS, min(iv_h, HEATK_STEPS) + 1, HEATK_N ** 3 * 4)},
            "heat_k_sqrt_n": {"forward_ms": tfh_s, "backward_ms": tbh_s, "backward_over_forward": tbh_s / tfh_s,
                              "forward_value": HEATK_N ** 3 * HEATK_STEPS / (tfh_s * 1e-3) / 1e9,
                              "checkpoints": kept(default_interval(HEATK_STEPS), HEATK_STEPS, 0)},
        }
        print(json.dumps(line), flush=True)


def reference_sg_gpu(workload: str, warmup: int) -> dict | None:
    """The reference's own single-GPU CUDA build on this GPU: its kernels compiled from its sources
    with its flags (-O3, FMA contraction on) into cubins, launched with its launch geometry (run.sh
    block sizes) in its host loop (oracle/ref_gpu.py). FP64, its only precision. Inputs come from the
    oracle's generators (this library is not loaded). None when the cubins or the GPU are absent."""
    try:
        import torch
        from oracle import ref_gpu
        if not torch.cuda.is_available() or not ref_gpu.available("heat3d"):
            return None
    except Exception:
        return None
    from oracle import oracle
    dev = torch.device("cuda:0")
    out = {"precision": "f64", "source": "reference kernels.cu compiled -O3 for sm_103a, reference launch geometry"}

    def timed(fn):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record()
        fn()
        ev1.record()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) * 1e-3

    n = 256
    if workload in ("heat3d", "heat2d", "ensemble"):
        mod = ref_gpu.RefModule("heat3d")
        from multigpu_advectiondiffusion_gb300.solvers import HeatConfig
        # the reference's constants for a 256^3 node grid on [0,10]^3 (main.cpp:55-62)
        base = HeatConfig.reference_3d(1.0, 10, 10, 10, n, n, n)
        k4, dt = base.kx, base.dt
        u = torch.from_numpy(oracle.ic_heat3d_blobs(n, n, n, 2)).to(dev)
        for _ in range(max(1, warmup)):
            ref_gpu.heat3d_run(mod, u, n, n, n, k4, k4, k4, dt, 2, block=(32, 4, 4), scheme="o2-euler")
        steps = 200
        t = timed(lambda: ref_gpu.heat3d_run(mod, u, n, n, n, k4, k4, k4, dt, steps, block=(32, 4, 4),
                                             scheme="o2-euler"))
        out["heat3d_256_o2_euler"] = {"value": n ** 3 * steps / t / 1e9, "unit": "Gcell-updates/s",
                                      "sample": f"{steps} forward-Euler steps (Compute_Laplace3d_O2 + Compute_RK, "
                                                "uo copy per step)"}
        steps = 20
        t = timed(lambda: ref_gpu.heat3d_run(mod, u, n, n, n, k4, k4, k4, dt, steps, block=(32, 4, 4)))
        out["heat3d_256_o4_rk3"] = {"value": n ** 3 * 3 * steps / t / 1e9, "unit": "Gcell-updates/s",
                                    "sample": f"{steps} SSP-RK3 steps of the baseline code"}
        mod.close()
    if workload in ("burgers3d", "ensemble"):
        mod = ref_gpu.RefModule("burgers3d")
        nb = 256
        dx = 2.0 / (nb - 1)
        u = torch.from_numpy(oracle.ic_burgers_ref(nb, nb, nb, dx, dx, dx)).to(dev)
        ref_gpu.burgers3d_run(mod, u, nb, 2.0, 1.0, 0.3, block=8, max_steps=1)
        steps = 3
        t = timed(lambda: ref_gpu.burgers3d_run(mod, u, nb, 2.0, 1.0, 0.3, block=8, max_steps=steps))
        out["burgers3d_256"] = {"value": nb ** 3 * 3 * steps / t / 1e9, "unit": "Gcell-updates/s",
                                "sample": f"{steps} SSP-RK3 steps (Compute_dF/dG/dH + Compute_Laplace_Async + "
                                          "Compute_RK per stage), local LF WENO5-Z, viscous, frozen layers"}
        mod.close()
    return out


def cpu_reference_sample(args, world: int, oracle):
    """A bounded sample of a non-heat workload run by the oracle's restatement on the host cores
    (test infrastructure: the reference has no CPU code for the path): per-step rates, seconds,
    a description of the sample and the workload's config."""
    if args.workload == "burgers3d":
        from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig
        n = 256
        cfg = BurgersConfig.periodic(n, weno=args.weno, div=args.div)
        u0 = ic_burgers_fourier(n, n, n, 2.0, 3, source="oracle").astype(np.float32)
        rates, secs = [], []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            _, _, it = oracle.burgers_run(cfg, u0, 10.0, 0.4, 1, max_steps=1, div64=args.div == "f64")
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                rates.append(cfg.numel * 3 * it / dt / 1e9)
                secs.append(dt)
        sample = f"256^3 FP32 WENO5-{args.weno.upper()} periodic, 1 of the 20 SSP-RK3 time steps per step (oracle)"
        config = burgers_config(args, world)
    elif args.workload == "adjoint":
        # the oracle's adjoint (stored states, OpenMP) on a 48^3 sample of the Burgers problem
        from multigpu_advectiondiffusion_gb300.solvers import BurgersConfig
        n = 48
        cfg = BurgersConfig(n, n, n, 2.0 / n, 2.0 / n, 2.0 / n, 1, 0, 1, 0)  # WENO5-Z, local LF, periodic
        u0 = ic_burgers_fourier(n, n, n, 2.0, 5, source="oracle")
        ut = ic_burgers_fourier(n, n, n, 2.0, 6, source="oracle")
        dt = 0.4 * cfg.dx / float(np.abs(u0).max())
        rates, secs = [], []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            oracle.burgers_loss_and_gradient(cfg, u0, ut, dt, 2)
            dt_ = time.perf_counter() - t0
            if i >= args.warmup:
                rates.append(n ** 3 * 3 * 2 / dt_ / 1e9)
                secs.append(dt_)
        sample = "48^3 FP64 WENO5-Z local LF periodic, 2 steps forward + adjoint per step (oracle)"
        config = adjoint_config(world)
    elif args.workload == "weno7":
        # the oracle's restatement of the prototype loop (FP64, OpenMP over lines) on a 96^3 sample,
        # one LSRK(5,4) step per benchmark step
        n = 96
        _, u0 = weno7_case(n)
        u0 = u0.reshape(n, n, n)
        h = 2.0 / (n - 1)
        rates, secs = [], []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            _, _, it = oracle.proto_run(7, u0, [h, h, h], 0.4, 1e9, max_steps=1)
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                rates.append(n ** 3 * 5 * it / dt / 1e9)
                secs.append(dt)
        sample = "96^3 FP64 WENO7 prototype scheme, 1 LSRK(5,4) step per step (oracle)"
        config = weno7_config(world)
    else:
        # the ensemble: per step, two heat instances for 4 steps and one Burgers instance for one
        # RK3 step, in proportion to the ensemble's heat / Burgers cell updates
        heat, burgers = ensemble_members()
        h0, b0 = ensemble_initial_states(heat[:2], burgers[:1], source="oracle")
        rates, secs = [], []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            cells = 0
            for c, a in zip(heat[:2], h0):
                oracle.cpu_heat_euler_o2(c, a.copy(), 4)
                cells += c.numel * 4
            _, _, it = oracle.burgers_run(burgers[0], b0[0], 1e9, 0.4, 1, max_steps=1, div64=False)
            cells += burgers[0].numel * 3 * it
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                rates.append(cells / dt / 1e9)
                secs.append(dt)
        sample = "2 heat instances x 4 Euler steps + 1 Burgers instance x 1 SSP-RK3 step of the ensemble"
        config = ensemble_config(world)
    return rates, secs, sample, config


def cpu_baseline_sample(args, world: int) -> dict:
    """cpu_baseline of a GPU line for a non-heat workload: the oracle on a bounded sample (one
    warm-up, two timed samples), all host threads."""
    from oracle import oracle
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    a = argparse.Namespace(**vars(args))
    a.warmup, a.steps = 1, 2
    rates, _, sample, _ = cpu_reference_sample(a, world, oracle)
    return {"value": float(np.median(rates)), "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
            "sample": sample, "cpu_model": cpu_model()}


def run_reference_arm(args, world, rank):
    """--impl reference: the path's CPU implementation on the host cores, for the same workload,
    metric and config as this library's line. The reference has no CPU code for the path, so this is
    its scheme restated (the tuned CPU loop for heat, the oracle otherwise), with the inputs from
    the oracle's generators; the library itself is not loaded. Each benchmark step is a bounded
    sample of the workload; ms_per_step is its measured wall time."""
    from oracle import oracle
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    if args.workload in ("heat3d", "heat2d"):
        cfg, nsteps = heat_case(args.workload)
        u0 = heat_initial(args.workload, source="oracle")
        budget = 4.0
        for _ in range(args.warmup):
            cpu_heat_rate(cfg, u0, nsteps, 0.2)
        rates, samples, secs = [], [], []
        for _ in range(args.steps):
            r, st, dt = cpu_heat_rate(cfg, u0, nsteps, budget)
            rates.append(r)
            samples.append(st)
            secs.append(dt)
        sample = (f"{cfg.nx}^{cfg.ndim} FP32 O2 Euler, {int(np.median(samples))} of the {nsteps} time steps per "
                  "step (tuned CPU loop, oracle/cpu_baseline.cpp, OpenMP)")
        config = heat_config(args.workload, world)
    else:
        rates, secs, sample, config = cpu_reference_sample(args, world, oracle)
    value = float(np.median(rates))
    line = {"impl": "reference", "metric": "Gcell-updates/s/RK-stage", "value": value, "unit": "Gcell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(secs)) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": config,
            "cpu_baseline": {"value": value, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
                             "sample": sample, "cpu_model": cpu_model()},
            "e2e": {"value": value, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "sg_gpu": reference_sg_gpu(args.workload, args.warmup)}
    print(json.dumps(line), flush=True)


WENO7_N, WENO7_STEPS = 256, 10


def weno7_case(n: int = WENO7_N):
    """The WENO7 prototype's problem (LFWENO7FDM3d.m): u0 = exp(-(x^2+y^2+z^2)/0.1) on the node grid
    of [-1,1]^3, CFL 0.4, here at n^3 FP32; (config, u0)."""
    from multigpu_advectiondiffusion_gb300.solvers import Weno7Config
    x = np.linspace(-1.0, 1.0, n)
    h = 2.0 / (n - 1)
    u0 = np.exp(-(x[None, None, :] ** 2 + x[None, :, None] ** 2 + x[:, None, None] ** 2) / 0.1).ravel()
    return Weno7Config(n, n, n, h, h, h), u0


def weno7_config(world: int) -> dict:
    return {"workload": f"weno7 {WENO7_N}^3 f32 (prototype scheme: local LF, clamped ends, LSRK(5,4)), gaussian, "
                        f"cfl 0.4 x {WENO7_STEPS} steps",
            "parallelism": f"replicas{world}",
            "l2": "per stage 4 sweeps of 64 MiB arrays > 126 MiB L2; 252 MiB L2 flush between GPU steps"}


# FP32 flops per cell-stage of the WENO7 right-hand side, counted from the ncu instruction mix of
# adv_weno7_rhs at 256^3 (FP32 state: the tiled face kernels with paired instructions and
# reciprocal-based weights). Per cell: FFMA2 153 x 4 + FADD2 21 x 2 + FMUL2 96 x 2 + FFMA 22.3 x 2
# + FADD 11.0 + FMUL 50.6 = 952.25. (The prototype's own operand order, which the FP64 state
# keeps, counted 1949: FFMA 495 x 2 + FADD 401 + FMUL 558.)
WENO7_FLOPS_PER_CELL_STAGE = 952.25


def bench_weno7(args, world, rank, dev, stream, flush, lib):
    """The WENO7 prototype solver at 256^3 FP32: one benchmark step = 10 LSRK(5,4) time steps (50
    stages) through adv_weno7_run; rel-L2 of a 0.05-time-unit run against the same run in FP64."""
    import torch
    from multigpu_advectiondiffusion_gb300.solvers import weno7_run, weno7_workspace
    cfg, u0n = weno7_case()
    u0 = torch.from_numpy(u0n.astype(np.float32)).to(dev)
    u = u0.clone()
    ws = weno7_workspace(cfg, u)
    sh = stream.cuda_stream
    S = WENO7_STEPS

    def one_step():
        weno7_run(cfg, u, 1e9, 0.4, max_steps=S, workspace=ws, stream=sh)

    def timed(fn, K):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(K):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1)

    for _ in range(args.warmup):
        u.copy_(u0)
        one_step()
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    u.copy_(u0)
    with ClockSampler(uuid) as clk:
        launches0 = lib.adv_kernel_launch_count()
        ms = timed(one_step, args.steps)
        launched = lib.adv_kernel_launch_count() - launches0
    ms_max = max_over_ranks(ms, dev)
    work = cfg.numel * 5 * S
    value = replica_throughput(work * args.steps, ms_max, world)
    # rooflines of one LSRK stage (the L2 flushes' own time subtracted): HBM with the 2N-storage
    # stage's algorithmic 16 B per cell (read u and r, write u and r), and the FP32 CUDA-core rate
    fl = timed(lambda: None, args.steps)
    stage_s = max(ms - fl, 1e-9) * 1e-3 / (args.steps * 5 * S)
    peak, peak_kind = _peaks()
    achieved = 16 * cfg.numel / stage_s / 1e9
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = sms * 128 * 2 * 2070.0 * 1e6 / 1e12
    flops = WENO7_FLOPS_PER_CELL_STAGE * cfg.numel / stage_s / 1e12
    roofline = {"bound": "hbm", "kernel": "weno7_face_fast_kernel + weno7_residual_kernel (3 axes per stage)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": None, "algorithmic_bytes_per_launch": 16 * cfg.numel, "avg_launch_us": stage_s * 1e6,
                "launch": "one LSRK stage (six kernels)"}
    roofline_alu = {"bound": "fp32", "achieved": flops, "peak": fp32_peak, "unit": "TFLOP/s",
                    "frac": flops / fp32_peak, "flops_per_cell_stage": WENO7_FLOPS_PER_CELL_STAGE,
                    "peak_source": f"nominal: {sms} SMs x 128 FP32 lanes x 2 flop x 2070 MHz"}
    # accuracy: FP32 vs FP64 over a short run from the initial state
    a32 = u0.clone()
    a64 = torch.from_numpy(u0n).to(dev)
    t32, it32 = weno7_run(cfg, a32, 0.05, 0.4, stream=sh)
    t64, it64 = weno7_run(cfg, a64, 0.05, 0.4, stream=sh)
    rel = (torch.linalg.vector_norm(a32.double() - a64) / torch.linalg.vector_norm(a64)).item()
    host_in = u0.cpu().pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()

    def e2e_step():
        with torch.cuda.stream(stream):
            u.copy_(host_in, non_blocking=True)
        one_step()
        with torch.cuda.stream(stream):
            host_out.copy_(u, non_blocking=True)
    e2e_step()
    ems = max_over_ranks(timed(e2e_step, args.steps), dev)
    nbytes = u.numel() * u.element_size()
    if rank == 0:
        line = {
            "metric": "Gcell-updates/s/RK-stage", "value": value, "unit": "Gcell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (the prototype's Gaussian initial state)", "config": weno7_config(world),
            "roofline": roofline, "roofline_alu": roofline_alu,
            "cpu_baseline": cpu_baseline_sample(args, world) if world == 1 else None,
            "e2e": {"value": replica_throughput(work * args.steps, ems, world), "unit": "Gcell-updates/s",
                    "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
            "gpu_launches": int(launched), "clocks": clk.summary(),
            "rel_l2_vs_fp64": rel, "rel_l2_vs_fp64_after": f"t = 0.05: {it32} FP32 steps, {it64} FP64 steps",
        }
        print(json.dumps(line), flush=True)


def compat_program_rates(n: int = 256) -> dict | None:
    """The reference's own single-GPU programs (their main.cpp + tools.cpp, unmodified) linked
    against this library's compatibility libraries (oracle/_ref/refmain_*), run on an n^3 grid with
    the reference's command line: the rate from the wall-time difference of two run lengths, so
    process start-up, the host initial condition and the copies cancel. FP64 (the programs' REAL).
    None when the programs were not built."""
    ref = ROOT / "oracle" / "_ref"
    out = {}

    def wall(argv):
        t0 = time.perf_counter()
        r = subprocess.run(argv, capture_output=True, text=True, timeout=600, cwd=str(ref))
        return time.perf_counter() - t0, r

    exe = ref / "refmain_burgers3d"
    if exe.exists():
        its, ts = [], []
        for tend in (0.005, 0.02):
            t, r = wall([str(exe), str(tend), "0.3", "2", "2", "2", str(n), str(n), str(n), "8", "8", "8"])
            m = re.search(r"iterations: ([0-9.eE+-]+)", r.stdout)
            if r.returncode != 0 or not m:
                return None
            its.append(int(float(m.group(1))))
            ts.append(t)
        out["burgers3d"] = {"value": n ** 3 * 3 * (its[1] - its[0]) / (ts[1] - ts[0]) / 1e9, "unit": "Gcell-updates/s",
                            "sample": f"{n}^3, {its[0]} vs {its[1]} SSP-RK3 steps of the reference scheme (local LF "
                                      "WENO5-Z + viscous term, frozen layers), FP64"}
    exe = ref / "refmain_heat3d"
    if exe.exists():
        ts = []
        for iters in (20, 60):
            t, r = wall([str(exe), "1.0", "10", "10", "10", str(n), str(n), str(n), str(iters), "32", "4", "4"])
            if r.returncode != 0:
                return None
            ts.append(t)
        out["heat3d_o4_rk3"] = {"value": n ** 3 * 3 * 40 / (ts[1] - ts[0]) / 1e9, "unit": "Gcell-updates/s",
                                "sample": f"{n}^3, 20 vs 60 SSP-RK3 steps of the reference's O4 heat scheme, FP64"}
    if out:
        out["how"] = ("the reference's main.cpp + tools.cpp linked unmodified against libadvdiff_compat_*; "
                      "compare with the reference arm's sg_gpu (its own kernels.cu on this GPU)")
    return out or None


DIV_LABEL = {"f32": "f32 (ieee: the f64 division's quotient rounded to f32, bit for bit)", "f64": "f64",
             "fast": "fast (reciprocal, <= 2 ulp)"}


def burgers_workload(args) -> str:
    return (f"burgers3d 256^3 f32 weno5-{args.weno} global-lf periodic cfl 0.4 x 20 steps, "
            f"div {DIV_LABEL[args.div]}")


def burgers_config(args, world: int) -> dict:
    return {"workload": burgers_workload(args), "parallelism": f"replicas{world}",
            "l2": "per stage 64 MiB read (+64 MiB for stages 2-3) + 64 MiB written > 126 MiB L2; "
                  "252 MiB L2 flush between GPU steps"}


def adjoint_config(world: int) -> dict:
    return {"workload": f"adjoint burgers3d {ADJ_N}^3 f32 weno5-z local-lf periodic, {ADJ_STEPS} steps to t={ADJ_T}, "
                        f"checkpoints by the default policy (the whole run kept in HBM when it fits; every "
                        f"{ADJ_INTERVAL} steps reported beside); heat k(x) {HEATK_N}^3 f32 {HEATK_STEPS} steps",
            "parallelism": f"replicas{world}"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="heat3d",
                    choices=["heat3d", "heat2d", "burgers3d", "weno7", "ensemble", "adjoint"])
    ap.add_argument("--cpu-budget", type=float, default=10.0, help="seconds of CPU-baseline work")
    ap.add_argument("--div", default="f64", choices=["fast", "f32", "f64"],
                    help="Burgers WENO weight division (FP32 state): f64 = computed in FP64 (the default); f32 = "
                         "IEEE FP32, equal bit for bit to the FP64 division rounded to the state; fast = "
                         "reciprocal-based")
    ap.add_argument("--weno", default="z", choices=["z", "js"], help="Burgers WENO5 flavour")
    ap.add_argument("--no-tune", action="store_true", help="skip the launch-shape autotuner")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl != "reference":
        prime_device(local)

    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return

    import torch
    import torch.distributed as dist
    from multigpu_advectiondiffusion_gb300 import _native as N
    from multigpu_advectiondiffusion_gb300.solvers import (BurgersConfig, autotune_burgers, autotune_heat, burgers_run,
                                                           burgers_workspace, heat_run, heat_workspace)

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

    if args.workload in ("ensemble", "adjoint", "weno7"):
        if args.workload == "ensemble":
            bench_ensemble(args, world, rank, dev, stream, flush, lib)
        elif args.workload == "weno7":
            bench_weno7(args, world, rank, dev, stream, flush, lib)
        else:
            bench_adjoint(args, world, rank, dev, lib)
        if world > 1:
            dist.destroy_process_group()
        return
    heat = args.workload in ("heat3d", "heat2d")
    if heat:
        cfg, inner = heat_case(args.workload)
        u0_np = heat_initial(args.workload)
        u0 = torch.from_numpy(u0_np).to(dev)
        u = u0.clone()
        ws = heat_workspace(cfg, u)
        cells_stages_per_step = cfg.numel * inner

        def one_step(uu):
            heat_run(cfg, uu, inner, ws, stream=sh)
        tuned = None if args.no_tune else autotune_heat(cfg, u, stream=sh)
        config = heat_config(args.workload, world)
        kernel = ("heat_stage_kernel<float,2,3,TMA,stage 1,4 rows,4 warps>" if cfg.ndim == 3
                  else "heat2d_multi_kernel<float,2,FMA> (up to 8 forward-Euler steps per launch, one read and "
                       "one write of the state per launch)")
    else:
        n = 256
        cfg = BurgersConfig.periodic(n, weno=args.weno, div=args.div)
        u0 = torch.from_numpy(ic_burgers_fourier(n, n, n, 2.0, 3).astype(np.float32)).to(dev)
        u = u0.clone()
        ws = burgers_workspace(cfg, u)
        inner = 20
        cells_stages_per_step = cfg.numel * 3 * inner

        def one_step(uu):
            burgers_run(cfg, uu, 1e9, 0.4, N.ADV_DT_MAXU, max_steps=inner, workspace=ws, stream=sh)
        tuned = None if args.no_tune else autotune_burgers(cfg, u, stream=sh)
        config = burgers_config(args, world)
        kernel = f"burgers_stage_kernel<float,{args.weno.upper()},{args.div} div>"

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
    settle(lambda: one_step(u))
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    with ClockSampler(uuid) as clk:
        settle(lambda: one_step(u), 1.0)  # the sampler's start-up (NVML) overlaps untimed work
        launches0 = lib.adv_kernel_launch_count()
        ms = timed(lambda: one_step(u), args.steps)
        launched = lib.adv_kernel_launch_count() - launches0
    # time of the L2 flushes alone, subtracted from the per-launch figure only
    fl = timed(lambda: None, args.steps)
    ms_max = max_over_ranks(ms, dev)
    value = replica_throughput(cells_stages_per_step * args.steps, ms_max, world)
    # stage launches of one benchmark step (Burgers: 3 per time step; its per-step dt kernel is
    # counted by the library but timed with the stages); each stage launch reads and writes the
    # state once, whatever number of time steps it advances
    if heat:
        launches_per_step = max(1, launched // max(1, args.steps))
        bytes_per_launch = 8 * cfg.numel
        if launches_per_step * 2 <= inner:  # the tuner chose two Euler steps per launch
            kernel = "heat_twostep_kernel (two forward-Euler steps per launch)"
    else:
        launches_per_step = inner * 3
        bytes_per_launch = (8 + 12 + 12) / 3 * cfg.numel
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
    ems = max_over_ranks(timed(e2e_step, args.steps), dev)
    e2e_value = replica_throughput(cells_stages_per_step * args.steps, ems, world)
    nbytes = u.numel() * u.element_size()

    # ---- accuracy of the FP32 result against FP64 (same device kernels, bit-exact with the oracle)
    extra = {}

    def ev_time(fn):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) * 1e-3

    if heat:
        u32 = u0.clone()
        u64 = u0.double()
        heat_run(cfg, u32, inner, stream=sh)
        heat_run(cfg, u64, inner, stream=sh)
        torch.cuda.synchronize()
        extra["rel_l2_vs_fp64"] = (torch.linalg.vector_norm(u32.double() - u64) / torch.linalg.vector_norm(u64)).item()
        extra["rel_linf_vs_fp64"] = ((u32.double() - u64).abs().max() / u64.abs().max()).item()
        u64_ref = u64.clone()
        ws64 = heat_workspace(cfg, u64)
        for _ in range(2):
            heat_run(cfg, u64, inner, ws64, stream=sh)
        extra["f64_value"] = cells_stages_per_step * 3 / ev_time(
            lambda: [heat_run(cfg, u64, inner, ws64, stream=sh) for _ in range(3)]) / 1e9
        # FP64 in the fused multiply-add form (adv_heat_desc.contract = 1), and its distance from the
        # reference's rounding after the whole solve
        cfg_c = dataclasses.replace(cfg, contract=True)
        u64c = u0.double()
        heat_run(cfg_c, u64c, inner, ws64, stream=sh)
        torch.cuda.synchronize()
        extra["f64_contracted_rel_l2_vs_f64"] = (torch.linalg.vector_norm(u64c - u64_ref) /
                                                 torch.linalg.vector_norm(u64_ref)).item()
        extra["f64_contracted_after"] = f"{inner} time steps from the same initial state"
        extra["f64_fast_value"] = cells_stages_per_step * 3 / ev_time(
            lambda: [heat_run(cfg_c, u64c, inner, ws64, stream=sh) for _ in range(3)]) / 1e9
    else:
        # ALU roofline: the stage is compute-bound. FP32 flops per cell-stage from the ncu
        # instruction mix of the stage kernel (FFMA2 = 4, FADD2/FMUL2/FFMA = 2, FADD/FMUL = 1);
        # peak = nominal FP32 CUDA-core rate.
        sm_mhz = 2070.0
        try:
            sm_mhz = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("sm_max_mhz", sm_mhz))
        except Exception:
            pass
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        fp32_peak = sms * 128 * 2 * sm_mhz * 1e6 / 1e12
        flops = BURGERS_FLOPS_PER_CELL_STAGE * cfg.numel / (launch_ms * 1e-3) / 1e12
        extra["roofline_alu"] = {"bound": "fp32", "kernel": kernel, "achieved": flops, "peak": fp32_peak,
                                 "unit": "TFLOP/s", "frac": flops / fp32_peak,
                                 "peak_source": f"nominal: {sms} SMs x 128 FP32 lanes x 2 flop x {sm_mhz:.0f} MHz",
                                 "flops_per_cell_stage": BURGERS_FLOPS_PER_CELL_STAGE}
        # the other WENO weight divisions on the same problem (one benchmark step each)
        others = {}
        for dv in ("fast", "f32", "f64"):
            if dv == args.div:
                continue
            c2 = BurgersConfig.periodic(256, weno=args.weno, div=dv)
            u2 = u0.clone()
            w2 = burgers_workspace(c2, u2)
            burgers_run(c2, u2, 1e9, 0.4, N.ADV_DT_MAXU, max_steps=2, workspace=w2, stream=sh)
            sec = ev_time(lambda: burgers_run(c2, u2, 1e9, 0.4, N.ADV_DT_MAXU, max_steps=inner, workspace=w2,
                                              stream=sh))
            others[dv] = cells_stages_per_step / sec / 1e9
            del u2, w2
        extra["other_division_values"] = others
        extra["compat_reference_programs"] = compat_program_rates()
        # the whole C3 run to t = 0.5 (past shock formation) in FP32 with this division and in FP64 in the
        # reference's operand order (bit-exact with the oracle): steps and relative L2 error
        u32 = u0.clone()
        t32, it32 = burgers_run(cfg, u32, 0.5, 0.4, N.ADV_DT_MAXU, workspace=ws, stream=sh)
        c64 = BurgersConfig.periodic(256, weno=args.weno, div="f32")
        u64 = u0.double()
        t64, it64 = burgers_run(c64, u64, 0.5, 0.4, N.ADV_DT_MAXU, stream=sh)
        extra["rel_l2_vs_fp64"] = (torch.linalg.vector_norm(u32.double() - u64) / torch.linalg.vector_norm(u64)).item()
        extra["rel_linf_vs_fp64"] = ((u32.double() - u64).abs().max() / u64.abs().max()).item()
        extra["rel_l2_vs_fp64_after"] = f"the run to t = 0.5: {it32} FP32 steps, {it64} FP64 steps"
        del u32
        # FP64 state, same problem: the reference's operand order (bit-exact with the oracle) and
        # the common-denominator form (ADV_DIV_FAST), two steps each
        for key, dv in (("f64_value", "f32"), ("f64_fast_value", "fast")):
            c64 = BurgersConfig.periodic(256, weno=args.weno, div=dv)
            u64 = u0.double()
            ws64 = burgers_workspace(c64, u64)
            burgers_run(c64, u64, 1e9, 0.4, N.ADV_DT_MAXU, max_steps=1, workspace=ws64, stream=sh)
            sec = ev_time(lambda: burgers_run(c64, u64, 1e9, 0.4, N.ADV_DT_MAXU, max_steps=2, workspace=ws64,
                                              stream=sh))
            extra[key] = cfg.numel * 3 * 2 / sec / 1e9
            del u64, ws64

    # ---- CPU baseline (the tuned CPU loop on the host cores, rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1:
        cpu = cpu_baseline_heat(cfg, u0_np, inner, args.cpu_budget) if heat else cpu_baseline_sample(args, world)

    if rank == 0:
        line = {
            "metric": "Gcell-updates/s/RK-stage", "value": value, "unit": "Gcell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Philox4x32-10 initial condition)",
            "config": config,
            "launch_shape": ({"ctas_per_sm": tuned["param_a"], "min_planes_per_cta": tuned["param_b"],
                              "tuned_us": tuned["best_us"], "default_us": tuned["default_us"]}
                             if tuned else "default"),
            "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "traffic": _traffic(args.workload),
                         "traffic_note": TRAFFIC_NOTE,
                         "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_us": launch_ms * 1e3,
                         "launches_per_step": launches_per_step},
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
