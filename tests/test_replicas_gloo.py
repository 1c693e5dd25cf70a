"""The multi-GPU path of the benchmark, on CPU: each rank runs an independent replica (the solvers
do not shard), the job's time is the slowest rank's and the value counts every rank's work. Two
gloo ranks on 127.0.0.1 run the same aggregation helpers bench.py uses; the reference arm prints
from rank 0 only."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [10.0, 25.0][rank]  # rank 1 is the slow replica
        ms_max = bench.max_over_ranks(ms)
        out[rank] = (ms_max, bench.replica_throughput(1e9, ms_max, world))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_replica():
    mp = pytest.importorskip("torch.multiprocessing")
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(world):
        ms_max, value = res[r]
        assert ms_max == 25.0
        assert value == pytest.approx(world * 1e9 / 25e-3 / 1e9)  # 80 G units/s for the job


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks(7.5) == 7.5
    assert bench.replica_throughput(2e9, 1000.0, 1) == pytest.approx(2.0)


def _ref_rank(rank, world, port, out):
    import contextlib
    import io
    import types

    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        buf = io.StringIO()
        if rank != 0:  # ranks other than 0 exit without work or output
            with contextlib.redirect_stdout(buf):
                bench.run_reference_arm(types.SimpleNamespace(workload="heat3d", steps=1, warmup=1), world, rank)
        out[rank] = buf.getvalue()
    finally:
        dist.destroy_process_group()


def test_reference_arm_other_ranks_print_nothing():
    mp = pytest.importorskip("torch.multiprocessing")
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_ref_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert out[1] == ""
