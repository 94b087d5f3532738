"""Benchmark harness logic on CPU: max-over-ranks timing over gloo (world size 2),
clock-record parsing, the roofline constants and the reference arm."""

import json
import math
import os
import subprocess
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from py4dstem_gb300 import roofline  # noqa: E402


def _rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)

    def reduce_max(x):
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    calls = []

    def step():
        calls.append(1)
        time.sleep(0.02 * (rank + 1))  # rank 1 is the slow one

    ms = bench.timed_region(step, 3, dist.barrier, lambda: None,
                            lambda: time.perf_counter() * 1e3, reduce_max)
    out.put((rank, ms, len(calls)))
    dist.destroy_process_group()


def test_timed_region_max_over_ranks_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    # every rank steps K times and reports the same (max) time, that of rank 1
    assert [r[2] for r in res] == [3, 3]
    assert res[0][1] == res[1][1]
    assert res[0][1] >= 3 * 0.04 * 1e3 * 0.95


def test_timed_region_single_rank_order():
    log = []
    ms = bench.timed_region(lambda: log.append("step"), 2, lambda: log.append("barrier"),
                            lambda: log.append("sync"), lambda: float(len(log)), lambda x: x)
    assert log == ["barrier", "sync", "step", "step", "sync", "barrier"]
    assert ms == 3.0  # now_ms read after the first sync and after the last


def test_clock_summary_parsing():
    s = bench.ClockSampler()
    s.lines = [
        "0, 1965, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2070, 2070, 1200.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2010, 2070, 1100.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    out = s.summary()
    assert out["sm_mhz"] == 2010 and out["sm_max_mhz"] == 2070
    assert out["reasons"] == ["sw_power_cap"] and out["samples"] == 3
    assert bench.ClockSampler().summary()["samples"] == 0


def test_roofline_constants():
    n = 128 * 128
    f = roofline.flops_per_position(n)
    assert math.isclose(f, 3 * 5 * n * 14 + 50 * n)
    assert math.isclose(f / 1e6, 4.26, rel_tol=2e-3)
    assert roofline.bytes_per_position(n) == 24 * n
    # multislice T=8 ~ 39 MFLOP, mixed M=4 ~ 16.1 MFLOP at 128^2
    assert math.isclose(roofline.flops_per_position(n, num_slices=8) / 1e6, 39.2, rel_tol=0.01)
    assert math.isclose(roofline.flops_per_position(n, num_probes=4) / 1e6, 16.1, rel_tol=0.01)
    # at the measured peaks the single-slice update sits at the ridge
    name, t = roofline.bound(f, 24 * n, 77.0, 6787.2)
    assert name == "hbm" and 50e-9 < t < 60e-9
    assert roofline.bound(f, 24 * n, 60.0, 6787.2)[0] == "fp32"


def test_bench_config_same_for_both_arms():
    a = bench.bench_config(128, 1024, [512, 512], 1)
    assert a["positions"] == 16384 and a["batch"] == 1024 and a["detector"] == 128


@pytest.mark.slow
def test_reference_arm_runs_on_cpu():
    out = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
         "--warmup", "0", "--ref-cores", "1"],
        capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["cores"] == 1 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["config"] == bench.bench_config(128, 1024, [512, 512], 1)
