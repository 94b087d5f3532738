"""Throughput benchmark of the GPU ptychography path (position updates/s).

Workload (default): single-slice gradient-descent ptychography at a 128^2
detector: 128x128 raster scan (J = 16384 positions, 0.75 A step), 512^2 object
at 0.25 A, 300 kV / 20 mrad / 100 A defocus probe, 1e5 e-/pattern, batch 1024.
Data are seeded synthetic patterns from py4dstem_gb300.synthetic (no public
dataset exists for this benchmark).

One step = one full reconstruction iteration over all J positions (16 batches
of 1024, per-iteration constraints and the error read-back the reference does
each iteration).

  value  device-resident amplitudes (1 GiB f32, larger than L2), K iterations
         timed with CUDA events between barriers;
  e2e    the public API: K calls of reconstruct(num_iter=1) on a
         SingleslicePtychography with storage="cpu" whose amplitudes live in
         page-locked host memory; each call uploads object, probe and positions,
         its kernels read all amplitudes from host memory over the CPU-GPU link,
         and it reads object, probe and error back;
  preprocess  preprocess() with the rotation search on the device for the whole
         scan, against the host NumPy path on a sample of scan rows.

Other workloads (--workload): multiscan (16 mixed-state scans in one graph
launch per iteration), multislice (8 slices), projection (DM_AP on whole-scan
batches), poscorr (position correction), mixed-multislice (4 slices, 2 modes),
tomography (8 tilts through a rotated 3D volume, 8 slices).

`--impl reference` times the reference algorithm (the float32 NumPy restatement
in oracle/, which reproduces the reference CPU path bit for bit) on the host
cores, one worker process per core, each step a bounded sample of batches.

Multi-GPU (torchrun): replicas only — each rank reconstructs its own scan;
value = positions of all ranks / max-over-ranks time.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "position updates/s (128^2 det)"
UNIT = "positions/s"
WORKLOAD = "single-slice GD, 128x128 scan (J=16384), 128^2 detector, 512^2 object, batch 1024"


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-preprocess-timing", action="store_true",
                    help="skip the device / host preprocess() timing")
    ap.add_argument("--preprocess-host-patterns", type=int, default=2048,
                    help="patterns in the host preprocess() timing sample")
    ap.add_argument("--scan", type=int, default=128, help="scan side (positions = scan^2)")
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-seconds", type=float, default=15.0)
    ap.add_argument("--ref-cores", type=int, default=0,
                    help="reference arm: limit the worker processes (0 = all host cores)")
    ap.add_argument("--workload", choices=["gd128", "multiscan", "multislice", "projection",
                                           "poscorr", "mixed-multislice", "gd256", "tomography",
                                           "learned-init"],
                    default="gd128",
                    help="gd128: the single-slice 128^2-detector workload (default); multiscan: "
                         "16 mixed-state scans of uneven sizes in one graph-captured launch")
    ap.add_argument("--scans", type=int, default=16, help="multiscan: number of scans")
    ap.add_argument("--ms-batch", type=int, default=256, help="multiscan: max_batch_size")
    ap.add_argument("--staged-batch", type=int, default=128, help="gd256: max_batch_size")
    ap.add_argument("--li-scans", type=int, default=20000,
                    help="learned-init: training scans (128x128 positions each)")
    ap.add_argument("--li-epochs", type=int, default=8, help="learned-init: training epochs")
    ap.add_argument("--li-seeds", type=int, default=8,
                    help="learned-init: held-out seeds evaluated (the full evaluation: 64)")
    ap.add_argument("--li-iterations", type=int, default=200,
                    help="learned-init: iterations of the plain run")
    ap.add_argument("--schedule", type=int, default=0,
                    help="128^2 kernel schedule: 0 default (3), 1 shared-memory passes by "
                         "the whole block, 2 register-resident, 3 shared-memory passes by "
                         "groups of warps")
    return ap.parse_args(argv)


# ------------------------------------------------------------------ distributed
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def timed_region(step, steps, barrier, sync, now_ms, reduce_max):
    """Barrier + sync on both sides of `steps` calls of step(); returns the
    max-over-ranks elapsed milliseconds. The callables make the harness testable
    on CPU (gloo) without a GPU."""
    barrier()
    sync()
    t0 = now_ms()
    for _ in range(steps):
        step()
    sync()
    t1 = now_ms()
    barrier()
    return reduce_max(t1 - t0)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0, period_ms=50):
        self.gpu_index = gpu_index
        self.period_ms = period_ms
        self.proc = None
        self.lines = []
        self.first = threading.Event()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # start the timed region only once sampling runs (bounded wait)
            self.first.wait(timeout=5.0)
            self.lines.clear()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())
            self.first.set()

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ workload
def roofline_constants(n_pixels):
    """Algorithmic flops and bytes of one single-slice GD position update."""
    from py4dstem_gb300 import roofline

    return roofline.flops_per_position(n_pixels), roofline.bytes_per_position(n_pixels)


def measured_hbm_gbs():
    """Measured HBM copy bandwidth of this GPU model (MEASURED_PEAKS.json), else
    the 6.8 TB/s fallback; returns (GB/s, source)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (copy)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s"


def set_schedule(schedule):
    """The 128^2 kernel schedule for this process (refused values raise)."""
    from py4dstem_gb300 import _native

    if _native.lib().ptycho_set_kernel_schedule(128, int(schedule)) < 0:
        raise SystemExit(_native.lib().ptycho_last_error().decode())


def read_profile_traffic():
    """DRAM bytes per launch of the position kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "position_kernel_128_gd.md")
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(r"dram_bytes_per_launch_scaled:\s*([0-9.eE+]+)", text)
    return float(m.group(1)) if m else None


# The reference's own reconstruct() on the benchmark scan (seed 1234), written by
# tests/golden/make_golden.py --size: the bench checks its first iterations
# against this error history.
PARITY_FIXTURE = os.path.join(ROOT, "tests", "golden", "size_ss_scan128_det128.npz")
PARITY_SEED = 1234


def build_case(scan, seed, device):
    """The benchmark scan. The 128 x 128 scan of seed 1234 is generated by the
    portable NumPy backend, the same counts the reference reconstructed for the
    parity fixture; other sizes and seeds use the faster torch backend."""
    from py4dstem_gb300 import synthetic

    portable = scan == 128 and seed == PARITY_SEED
    case = synthetic.make_scan(
        "bench", seed, (scan, scan), 0.75, 0.05, 128, 512 if scan >= 128 else
        int(2 ** math.ceil(math.log2(scan * 3 + 128))), dose=1e5,
        backend="portable" if portable else "torch", device=device)
    return case


def parity_check(case, batch):
    """Three iterations of the public API on the benchmark scan against the
    reference's error history for the same data, seed and batch size (the
    fixture). Returns None when the fixture does not describe this workload."""
    if not os.path.exists(PARITY_FIXTURE) or batch != 1024:
        return None
    z = np.load(PARITY_FIXTURE)
    meta = json.loads(str(z["meta"]))
    gen = meta["generator"]
    if (gen["seed"] != PARITY_SEED or tuple(gen["scan_shape"]) != (128, 128)
            or not np.array_equal(case.scan_positions_ang, z["scan_positions_ang"])):
        return None
    import hashlib

    counts = np.ascontiguousarray(case.datacube.data.astype(np.uint16))
    if hashlib.sha256(counts.tobytes()).hexdigest() != meta["counts_digest"]:
        return {"ok": False, "reason": "the generated counts differ from the reference's input"}
    ref_err = np.asarray(z["out_error_iterations"], dtype=np.float64)
    p = preprocess(case, storage="gpu")
    p.reconstruct(progress_bar=False, **meta["reconstruct"])
    err = np.asarray(p.error_iterations, dtype=np.float64)
    d = float(np.max(np.abs(err - ref_err) / ref_err))
    # the reference's own rounding floor on this workload (FFTs through complex128)
    floor = float(meta["stats"]["floor_err"])
    tol = max(1e-5, 3.0 * floor)
    return {"iterations": len(err), "errors": err.tolist(), "reference_errors": ref_err.tolist(),
            "max_rel_diff": d, "reference_floor": floor, "tolerance": tol, "ok": bool(d <= tol),
            "reference": "reference reconstruct() on the same counts, seed and batch "
                         "(tests/golden/size_ss_scan128_det128.npz)"}


def preprocess(case, storage, device="gpu"):
    from py4dstem_gb300 import SingleslicePtychography

    kw = dict(case.ctor_kwargs)
    p = SingleslicePtychography(datacube=case.datacube, verbose=False, device=device,
                                storage=storage, **kw)
    p.preprocess(max_batch_size=1024, **case.preprocess_kwargs)
    return p


def preprocess_timing(case, host_patterns):
    """preprocess() with the rotation search (no forced rotation): on the device
    for the whole scan (wall time, synchronised; the library is already loaded),
    and the host NumPy path (device="cpu") on the first scan rows holding about
    `host_patterns` patterns, scaled to the whole scan by the pattern count."""
    import torch

    from py4dstem_gb300 import DataCube, SingleslicePtychography

    pre_kw = {k: v for k, v in case.preprocess_kwargs.items()
              if k not in ("force_com_rotation", "force_com_transpose")}
    kw = dict(case.ctor_kwargs)

    def run(datacube, positions, device):
        c = dict(kw, initial_scan_positions=positions)
        p = SingleslicePtychography(datacube=datacube, verbose=False, device=device,
                                    storage="gpu" if device == "gpu" else "cpu", **c)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p.preprocess(max_batch_size=1024, **pre_kw)
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    data = case.datacube.data
    rx, ry = data.shape[:2]
    J = rx * ry
    dev_s = run(case.datacube, case.scan_positions_ang, "gpu")
    rows = max(3, min(rx, host_patterns // ry))
    sub = DataCube(np.ascontiguousarray(data[:rows]), r_pixel_size=case.datacube.calibration
                   .get_R_pixel_size(), r_pixel_units="A",
                   q_pixel_size=case.datacube.calibration.get_Q_pixel_size(), q_pixel_units="mrad")
    n_host = rows * ry
    host_s = run(sub, case.scan_positions_ang[:n_host], "cpu")
    return {"device_s": dev_s, "patterns": J, "host_sample_s": host_s,
            "host_sample_patterns": n_host, "host_s_scaled": host_s * J / n_host,
            "speedup_vs_host_scaled": host_s * J / n_host / dev_s,
            "steps": "intensities upload, centre of mass, plane fit, rotation search "
                     "(179 angles x 2), corner-centring + sqrt, probe, probe overlap + FOV mask"}


def fp32_peak_tflops(torch, lib):
    """Measured FP32 FMA throughput of this GPU (TFLOP/s)."""
    import ctypes

    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    blocks = props.multi_processor_count * 8
    iters = 1 << 15
    sink = torch.empty(blocks * 256, dtype=torch.float32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        lib.ptycho_fp32_fma_probe(blocks, iters, ctypes.c_void_p(sink.data_ptr()), stream)
    best = 0.0
    for _ in range(5):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        lib.ptycho_fp32_fma_probe(blocks, iters, ctypes.c_void_p(sink.data_ptr()), stream)
        e.record()
        e.synchronize()
        ms = s.elapsed_time(e)
        best = max(best, 16.0 * blocks * 256 * iters / (ms * 1e-3) / 1e12)
    return best


def cpu_baseline_sample(p, seconds):
    """Oracle (reference algorithm, float32 NumPy) on one core: whole batches of the
    same workload until ~`seconds` of CPU work; positions/s."""
    from oracle.ptycho_np import Oracle, State

    st = State(amplitudes=p._amplitudes, positions_px=p._positions_px.copy(),
               probe=np.array(p._probe), object=np.array(p._object),
               mean_intensity=p._mean_diffraction_intensity,
               fov_mask_inverse=p._object_fov_mask_inverse)
    o = Oracle(st)
    J = p._num_diffraction_patterns
    B = min(1024, J)
    order = np.random.default_rng(0).permutation(J)
    done = 0
    t0 = time.perf_counter()
    sub = 128  # positions per sub-step, the timing granule
    while time.perf_counter() - t0 < seconds:
        idx = order[(done % J):(done % J) + sub]
        _run_oracle_batch(o, idx)
        done += len(idx)
    dt = time.perf_counter() - t0
    return done / dt, done, B


def _run_oracle_batch(o, idx):
    pos = o.positions_px[idx]
    frac = pos - np.round(pos)
    rows, cols = o.patch_indices(pos)
    shifted = o.fft_shift(o.probe, frac)
    shifted, patches, ov = o.overlap(rows, cols, shifted)
    ew, _ = o.gd_projection(o.amplitudes[idx], ov, None)
    o.adjoint(patches, shifted, pos, ew, 0.5, 1.0, False, False)


def _ms_ref_batch(state):
    """One gradient-descent batch of the mixed-state reference algorithm (float32
    NumPy restatement) on one core: (positions, seconds)."""
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"
    from oracle.ptycho_np import Oracle, State

    o = Oracle(State(**state))
    idx = np.arange(o.J)
    t0 = time.perf_counter()
    _run_oracle_batch(o, idx)
    return o.J, time.perf_counter() - t0


def multiscan_cpu_baseline(scans, batch):
    """The reference algorithm on the multi-scan workload: one batch of each scan
    (its first `batch` positions in a seeded order), the scans in parallel in
    single-threaded worker processes, one per host core as the scans allow;
    positions/s = sampled positions / the slowest worker's time."""
    import multiprocessing as mp

    states = []
    rng = np.random.default_rng(0)
    for p in scans:
        J = p._num_diffraction_patterns
        idx = np.sort(rng.permutation(J)[:min(batch, J)])
        amps = p._amplitudes_for_state()
        amps = amps[idx].cpu().numpy() if hasattr(amps, "cpu") else np.asarray(amps)[idx]
        states.append(dict(
            amplitudes=np.ascontiguousarray(amps, dtype=np.float32),
            positions_px=np.asarray(p._positions_px)[idx].astype(np.float32),
            probe=np.array(p._probe), object=np.array(p._object),
            mean_intensity=p._mean_diffraction_intensity,
            fov_mask_inverse=p._object_fov_mask_inverse, num_probes=p._num_probes, mixed=True))
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    workers = max(1, min(cores, len(states)))
    with mp.get_context("spawn").Pool(workers) as pool:
        res = pool.map(_ms_ref_batch, states, chunksize=1)
    n = sum(r[0] for r in res)
    # a worker runs its scans one after another: the slowest worker's sum of times
    per_worker = [0.0] * workers
    for k, r in enumerate(res):
        per_worker[k % workers] += r[1]
    return {"value": n / max(per_worker), "unit": UNIT, "cores": workers, "kind": "port",
            "sample": f"one batch of up to {batch} positions of each of the {len(states)} "
                      f"scans (float32 NumPy restatement of the reference's mixed-state "
                      f"gradient descent), {workers} single-threaded processes"}


def bench_config(scan, batch, object_shape, world):
    return {"workload": WORKLOAD, "positions": scan * scan, "batch": min(batch, scan * scan),
            "detector": 128, "object": object_shape, "iterations_per_step": 1,
            "l2": "inputs larger than L2 (1 GiB amplitudes)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


# ------------------------------------------------------------------ reference arm
_REF = {}


REF_SCAN = 32  # positions per worker: one batch of 1024


def _ref_init(seed):
    """Pool initializer: each worker process preprocesses (host NumPy path) its
    own 32 x 32 part of the benchmark workload: 0.75 A step, 128^2 detector, the
    512^2 object at 0.25 A, 1e5 e-/pattern; 1024 positions = one batch of 1024."""
    from py4dstem_gb300 import synthetic
    from oracle.ptycho_np import Oracle, State

    seed = seed + os.getpid() % 1000
    case = synthetic.make_scan("ref", seed, (REF_SCAN, REF_SCAN), 0.75, 0.05, 128, 512,
                               dose=1e5, backend="numpy")
    p = preprocess(case, storage="cpu", device="cpu")  # host NumPy preprocess
    st = State(amplitudes=p._amplitudes, positions_px=p._positions_px.copy(),
               probe=np.array(p._probe), object=np.array(p._object),
               mean_intensity=p._mean_diffraction_intensity,
               fov_mask_inverse=p._object_fov_mask_inverse)
    _REF["oracle"] = Oracle(st)
    _REF["order"] = np.random.default_rng(seed).permutation(p._num_diffraction_patterns)


def _ref_step(seconds):
    """Whole gradient-descent batches of 1024 positions on the 512^2 object (the
    benchmark's batch size and object) for at least `seconds`."""
    o, order = _REF["oracle"], _REF["order"]
    done = 0
    t0 = time.perf_counter()
    while True:
        _run_oracle_batch(o, order)
        done += len(order)
        if time.perf_counter() - t0 >= seconds:
            break
    return done, time.perf_counter() - t0


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import multiprocessing as mp

    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    if args.ref_cores:
        cores = min(cores, args.ref_cores)
    # NumPy's FFT, bincount and elementwise loops run on one thread; one worker
    # process per host core, each on one thread
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"
    per_step = max(1.0, min(20.0, 60.0 / max(1, args.steps + args.warmup)))
    ctx = mp.get_context("spawn")
    values = []
    with ctx.Pool(cores, initializer=_ref_init, initargs=(100,)) as pool:
        for i in range(args.warmup + args.steps):
            res = pool.map(_ref_step, [per_step] * cores, chunksize=1)
            tot = sum(r[0] for r in res)
            wall = max(r[1] for r in res)
            if i >= args.warmup:
                values.append(tot / wall)
    v = float(statistics.median(values))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * 16384 / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": bench_config(args.scan, args.batch, [512, 512] if args.scan >= 128 else None,
                               args.gpus),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} single-threaded processes (nproc {os.cpu_count()}), "
                                   f"each >= {per_step:.1f} s per step of whole 1024-position "
                                   "GD batches (128^2 detector, 512^2 object) of the float32 "
                                   "NumPy restatement of the reference"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ our arm
def run_ours(args):
    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        barrier = dist.barrier

        def reduce_max(x):
            t = torch.tensor([x], dtype=torch.float64, device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
    else:
        def barrier():
            return None

        def reduce_max(x):
            return x

    from py4dstem_gb300 import _native, engine

    lib = _native.lib()
    set_schedule(args.schedule)
    seed = 1234 + rank
    t_setup = time.time()
    case = build_case(args.scan, seed, f"cuda:{local}")
    p = preprocess(case, storage="gpu")
    setup_s = time.time() - t_setup
    pre_timing = None
    if rank == 0 and world == 1 and not args.no_preprocess_timing:
        pre_timing = preprocess_timing(case, args.preprocess_host_patterns)

    # CPU baseline on rank 0 at N=1 only, before any timing (single core)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, done, _ = cpu_baseline_sample(p, args.cpu_sample_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{done} positions of the same 128^2-detector GD workload "
                         "(float32 NumPy restatement of the reference, 1 core)"}

    J = p._num_diffraction_patterns
    B = min(args.batch, J)
    st = engine.create_state(
        roi_shape=tuple(p._region_of_interest_shape), object_array=np.asarray(p._object),
        probe_array=p._probe, amplitudes=p._amplitudes_for_state(),
        positions_px=p._positions_px,
        num_slices=1, num_probes=1, potential=False, max_batch=B, storage="gpu",
        fov_mask_inverse=p._object_fov_mask_inverse)
    driver_kw = dict(max_batch=B, step_size=0.5, normalization_min=1.0,
                     use_mask=bool(p._object_fov_mask_inverse.sum() > 0),
                     mean_intensity=p._mean_diffraction_intensity)
    # each iteration replays one CUDA graph of all its kernels (captured during
    # the warm-up)
    drv = engine.IterationDriver(st, graph=True, **driver_kw)
    np.random.seed(seed)
    order = np.arange(J)
    errors = []

    np.random.shuffle(order)

    def step(d=drv):
        d.iterate(order)
        np.random.shuffle(order)  # the next iteration's order, while the GPU works
        errors.append(float(d.error()))  # per-iteration read-back, as the reference

    for _ in range(max(args.warmup, 2)):
        step()
    torch.cuda.synchronize()
    import ctypes

    launches0 = st.launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)

    def now_ms():
        return time.perf_counter() * 1e3

    with ClockSampler(local) as clocks:
        ev0.record()
        wall_ms = timed_region(step, args.steps, barrier, torch.cuda.synchronize, now_ms,
                               lambda x: x)
        ev1.record()
        torch.cuda.synchronize()
    dev_ms = ev0.elapsed_time(ev1)
    ms = reduce_max(dev_ms)
    launches = st.launches - launches0
    # position-kernel time: CUDA events around each launch, in two more
    # iterations issued without the graph (outside the timed region)
    ms_dummy = ctypes.c_float()
    n_dummy = ctypes.c_int32()
    lib.ptycho_kernel_timing(ctypes.byref(ms_dummy), ctypes.byref(n_dummy))  # clear
    lib.ptycho_enable_kernel_timing(1)
    drv_t = engine.IterationDriver(st, graph=False, **driver_kw)
    for _ in range(2):
        step(drv_t)
    torch.cuda.synchronize()
    lib.ptycho_enable_kernel_timing(0)
    kms = ctypes.c_float()
    kn = ctypes.c_int32()
    _native.check(lib.ptycho_kernel_timing(ctypes.byref(kms), ctypes.byref(kn)))

    value = world * J * args.steps / (ms * 1e-3)
    flops_pos, bytes_pos = roofline_constants(128 * 128)
    kernel_avg_ms = kms.value / max(1, kn.value)
    nb = len(list(engine.generate_batches(J, B)))
    pos_per_launch = J / nb
    kernel_s = kernel_avg_ms * 1e-3
    fp32_peak = fp32_peak_tflops(torch, lib) if rank == 0 else None
    hbm_peak, hbm_source = measured_hbm_gbs()
    traffic = read_profile_traffic()
    fp32_achieved = flops_pos * pos_per_launch / kernel_s / 1e12
    hbm_achieved = bytes_pos * pos_per_launch / kernel_s / 1e9
    from py4dstem_gb300 import roofline as _rl

    bound_name, _ = _rl.bound(flops_pos, bytes_pos, fp32_peak or 77.0, hbm_peak)
    kernel_name = {1: "position_kernel<128,128,1024,1>", 2: "gd128_kernel"}.get(
        args.schedule, "position_grouped_kernel<1024>")
    if bound_name == "hbm":
        roof = {"bound": "hbm", "achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": hbm_achieved / hbm_peak, "peak_source": hbm_source + ", of measured"}
    else:
        roof = {"bound": "fp32", "achieved": fp32_achieved, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": fp32_achieved / fp32_peak if fp32_peak else None,
                "peak_source": "FP32 FMA probe measured live (ptycho_fp32_fma_probe), of measured"}
    roof.update({
        "traffic": traffic, "kernel": kernel_name, "kernel_avg_ms": kernel_avg_ms,
        "kernel_launches": kn.value, "positions_per_launch": pos_per_launch,
        "flops_per_position": flops_pos, "bytes_per_position": bytes_pos,
        "other_roofline": ({"bound": "fp32", "achieved": fp32_achieved, "peak": fp32_peak,
                            "unit": "TFLOP/s",
                            "frac": fp32_achieved / fp32_peak if fp32_peak else None}
                           if bound_name == "hbm" else
                           {"bound": "hbm", "achieved": hbm_achieved, "peak": hbm_peak,
                            "unit": "GB/s", "frac": hbm_achieved / hbm_peak}),
        "traffic_source": "ncu dram__bytes_read+write of one launch "
                          "(profiles/position_kernel_128_gd.md)",
    })

    # e2e through the public API with host-resident inputs
    e2e = None
    if not args.no_e2e:
        pe = p  # preprocessed above; the engine run did not modify its host state
        # amplitudes in page-locked host memory, storage="cpu": every step all of
        # them cross the CPU-GPU link, each batch's patterns gathered to the
        # device while the batch before it computes
        pe._amplitudes = torch.from_numpy(np.ascontiguousarray(pe._amplitudes)).pin_memory().numpy()
        pe._storage = "cpu"
        rec = dict(max_batch_size=B, seed_random=seed, progress_bar=False)
        for _ in range(max(1, args.warmup)):
            pe.reconstruct(num_iter=1, **rec)
        torch.cuda.synchronize()
        e_ms = timed_region(lambda: pe.reconstruct(num_iter=1, **rec), args.steps, barrier,
                            torch.cuda.synchronize, now_ms, reduce_max)
        h2d = int(pe._amplitudes.nbytes + np.asarray(pe._object).nbytes +
                  np.asarray(pe._probe).nbytes + pe._positions_px.nbytes)
        # the object twice (the working copy and the result attribute), probe, error
        d2h = int(2 * np.asarray(pe._object).nbytes + np.asarray(pe._probe).nbytes + 4)
        e2e = {"value": world * J * args.steps / (e_ms * 1e-3), "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "mode": "reconstruct(num_iter=1) per step, storage='cpu': amplitudes in "
                       "page-locked host memory, each batch's patterns gathered to the "
                       "device one batch ahead on a second stream"}

    parity = parity_check(case, B) if rank == 0 and args.scan == 128 else None

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": bench_config(args.scan, B, list(np.shape(p._object)), world),
            "iterations_per_s": args.steps / (ms * 1e-3),
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clocks.summary(),
            "final_error": errors[-1] if errors else None,
            "parity": parity,
            "setup_s": setup_s,
            "preprocess": pre_timing,
            "wall_ms_timed": wall_ms,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


# ------------------------------------------------------------------ multi-scan
def run_multiscan(args):
    """16 independent mixed-state scans (grids 24^2..96^2, detectors 64/96/128,
    M = 4, 1e4 e-/pattern) reconstructed in one graph-captured, concurrent launch
    per iteration; value = position updates/s over all scans. The same scans
    reconstructed one after another without a graph give `sequential_value`."""
    rank, world, local = dist_env()
    if world > 1:
        print(json.dumps({"workload": "multiscan", "unavailable": "single-GPU workload"}))
        return 0
    import torch

    torch.cuda.set_device(local)
    from py4dstem_gb300 import MixedstatePtychography, synthetic
    from py4dstem_gb300.multiscan import MultiScanReconstruction

    cases = synthetic.multiscan_cases(seed=7, num_scans=args.scans, backend="torch",
                                      device=f"cuda:{local}")
    scans = []
    for c in cases:
        kw = dict(c.ctor_kwargs)
        kw["initial_probe_guess"] = c.probe_modes.astype(np.complex64)
        p = MixedstatePtychography(datacube=c.datacube, verbose=False, device="gpu", **kw)
        p.preprocess(max_batch_size=args.ms_batch, **c.preprocess_kwargs)
        scans.append(p)
    J = sum(p._num_diffraction_patterns for p in scans)

    def timed(run, steps):
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        run.reconstruct(steps)
        t1.record()
        t1.synchronize()
        return t0.elapsed_time(t1)

    graph_run = MultiScanReconstruction(scans, max_batch_size=args.ms_batch, seed_random=1)
    graph_run.reconstruct(max(2, args.warmup))  # builds, tunes, captures
    with ClockSampler(local) as clocks:
        ms = timed(graph_run, args.steps)
    seq_run = MultiScanReconstruction(scans, max_batch_size=args.ms_batch, seed_random=1,
                                      use_graph=False, concurrent=False)
    seq_run.reconstruct(max(1, args.warmup))
    ms_seq = timed(seq_run, args.steps)
    line = {
        "metric": "position updates/s (16 mixed-state scans, M=4, one launch per iteration)",
        "value": J * args.steps / (ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "multiscan", "scans": [
            [int(round(np.sqrt(p._num_diffraction_patterns))),
             int(p._region_of_interest_shape[0])] for p in scans],
            "positions": J, "batch": args.ms_batch, "modes": 4, "iterations_per_step": 1},
        "sequential_value": J * args.steps / (ms_seq * 1e-3),
        "cpu_baseline": None if args.no_cpu_baseline else multiscan_cpu_baseline(
            scans, args.ms_batch),
        "tuning": {"choice": graph_run.tuning["choice"],
                   "timings_ms": [[c["concurrent"], t] for c, t in
                                  graph_run.tuning["timings_ms"]]},
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ multislice
def run_multislice(args):
    """The multislice workload: 8 slices of 20 A, 64x64 scan at 0.4 A, 128^2
    detector, 300 kV, 25 mrad, defocus 50 A, GD with batch 256; value = position
    updates/s (one step = one full iteration, device-resident amplitudes)."""
    rank, world, local = dist_env()
    if world > 1:
        print(json.dumps({"workload": "multislice", "unavailable": "single-GPU workload"}))
        return 0
    import torch

    torch.cuda.set_device(local)
    from py4dstem_gb300 import MultislicePtychography, engine, roofline, synthetic

    set_schedule(args.schedule)

    c = synthetic.multislice_case(seed=3, num_slices=8, scan=64, backend="torch",
                                  device=f"cuda:{local}", object_px=256)
    p = MultislicePtychography(datacube=c.datacube, verbose=False, device="gpu",
                               **c.ctor_kwargs)
    p.preprocess(max_batch_size=256, **c.preprocess_kwargs)
    J = p._num_diffraction_patterns
    B = 256
    st = engine.create_state(
        roi_shape=tuple(p._region_of_interest_shape), object_array=np.asarray(p._object),
        probe_array=p._probe, amplitudes=p._amplitudes, positions_px=p._positions_px,
        num_slices=p._num_slices, num_probes=1, potential=False, max_batch=B, storage="gpu",
        propagators=p._propagator_arrays,
        fov_mask_inverse=p._object_fov_mask_inverse)
    drv = engine.IterationDriver(st, max_batch=B, step_size=0.5, normalization_min=1.0,
                                 use_mask=bool(p._object_fov_mask_inverse.sum() > 0),
                                 mean_intensity=p._mean_diffraction_intensity)
    rng = np.random.RandomState(3)
    order = np.arange(J)

    rng.shuffle(order)

    def step():
        drv.iterate(order)
        rng.shuffle(order)
        drv.error()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        ev0.record()
        for _ in range(args.steps):
            step()
        ev1.record()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    n = 128 * 128
    line = {
        "metric": "position updates/s (multislice T=8, 128^2 det)",
        "value": J * args.steps / (ms * 1e-3), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "multislice", "slices": 8, "positions": J, "batch": B,
                   "detector": 128, "object": list(np.shape(p._object))},
        "flops_per_position": roofline.flops_per_position(n, num_slices=8),
        "achieved_tflops": roofline.flops_per_position(n, num_slices=8) * J * args.steps
        / (ms * 1e-3) / 1e12,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_variant(args):
    """The benchmark scan (128x128 positions, 128^2 detector, 512^2 object) with
    one of the options the reference runs at scale:
      projection        DM_AP (a=-1, b=1, c=2) on whole-scan batches (the
                        reference allows no mini-batches with projection sets),
                        2 GiB of persistent exit waves;
      poscorr           gradient descent, batch 1024, position correction with
                        both distance limits and the positions CoM constraint;
      mixed-multislice  a 64x64 scan through 4 slices with 2 probe modes, batch 256;
      gd256             gradient descent on a 256^2 detector (the staged batch-wide
                        kernels): a 64x64 scan at 0.75 A, 512^2 object, batch 128
                        (--staged-batch).
    value = position updates/s over K full iterations (device-resident amplitudes)."""
    rank, world, local = dist_env()
    if world > 1:
        print(json.dumps({"workload": args.workload, "unavailable": "single-GPU workload"}))
        return 0
    import torch

    torch.cuda.set_device(local)
    from py4dstem_gb300 import engine, roofline, synthetic
    from py4dstem_gb300.ptychography import method_parameters

    set_schedule(args.schedule)
    w = args.workload
    det = 256 if w == "gd256" else 128
    n = det * det
    if w == "gd256":
        case = synthetic.make_scan("ss256", 7, (64, 64), 0.75, 0.05, 256, 512, dose=1e5,
                                   backend="torch", device=f"cuda:{local}")
        p = preprocess(case, storage="gpu")
        B, T, M = args.staged_batch, 1, 1
    elif w == "mixed-multislice":
        from py4dstem_gb300 import MixedstateMultislicePtychography

        case = synthetic.make_scan("mms", 5, (64, 64), 0.4, 0.05, 128, 256, dose=1e5,
                                   num_slices=4, slice_thickness=20.0, num_modes=2,
                                   mode_weights=(0.8, 0.2), backend="torch",
                                   device=f"cuda:{local}")
        p = MixedstateMultislicePtychography(datacube=case.datacube, verbose=False,
                                             device="gpu", **case.ctor_kwargs)
        p.preprocess(max_batch_size=256, **case.preprocess_kwargs)
        B, T, M = 256, 4, 2
    else:
        case = build_case(128, 1234, f"cuda:{local}")
        p = preprocess(case, storage="gpu")
        B = p._num_diffraction_patterns if w == "projection" else 1024
        T, M = 1, 1
    J = p._num_diffraction_patterns
    projection = w == "projection"
    use_projection, pa, pb, pc, _, step = method_parameters(
        "DM_AP" if projection else "GD", 1.0, None, None, None, 0.5)
    poscorr = w == "poscorr"
    st = engine.create_state(
        roi_shape=tuple(p._region_of_interest_shape), object_array=np.asarray(p._object),
        probe_array=p._probe, amplitudes=p._amplitudes_for_state(),
        positions_px=p._positions_px, num_slices=T, num_probes=M, potential=False,
        max_batch=B, storage="gpu",
        propagators=p._propagator_arrays if T > 1 else None,
        fov_mask_inverse=p._object_fov_mask_inverse, projection=projection,
        mixed_state=M > 1, positions_initial=p._positions_px_initial if poscorr else None)
    drv = engine.IterationDriver(
        st, max_batch=B, projection=projection, projection_abc=(pa or 0, pb or 0, pc or 0),
        step_size=step, normalization_min=1.0,
        use_mask=bool(p._object_fov_mask_inverse.sum() > 0), orthogonalize_probe=M > 1,
        mean_intensity=p._mean_diffraction_intensity, graph=not poscorr,
        position_correction=(dict(step_size=0.9, max_update_px=0.5, max_total_px=2.0,
                                  center_of_mass=True) if poscorr else None))
    rng = np.random.RandomState(3)
    order = np.arange(J)

    def step_fn():
        if not projection:
            rng.shuffle(order)
        drv.iterate(order)
        drv.error()

    for _ in range(max(args.warmup, 2)):
        step_fn()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        ev0.record()
        for _ in range(args.steps):
            step_fn()
        ev1.record()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    fl = roofline.flops_per_position(n, num_slices=T, num_probes=M)
    line = {
        "metric": f"position updates/s ({w}, {det}^2 det)",
        "value": J * args.steps / (ms * 1e-3), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": max(args.warmup, 2), "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": w, "positions": J, "batch": B, "slices": T, "modes": M,
                   "detector": det, "object": list(np.shape(p._object)),
                   "method": "DM_AP" if projection else "GD",
                   "position_correction": poscorr},
        "flops_per_position": fl,
        "achieved_tflops": fl * J * args.steps / (ms * 1e-3) / 1e12,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def tilt_matrix(deg):
    """Rotation by `deg` degrees about the x (first, vertical) axis in (x, y, z)."""
    t = np.deg2rad(deg)
    return np.array([[1.0, 0.0, 0.0], [0.0, np.cos(t), -np.sin(t)],
                     [0.0, np.sin(t), np.cos(t)]])


def run_tomography(args):
    """Joint ptychographic tomography: 8 tilts (-35 to 35 degrees about x), each
    a 32x32 scan on a 64^2 detector, 8 slices through the rotated potential
    volume, batch 256, collective updates, gradient descent. value = position
    updates/s over K full iterations (every tilt: volume rotation, projection,
    the multislice batches, update expansion and back-rotation), timed around
    one reconstruct(num_iter=K) call with device-resident amplitudes."""
    rank, world, local = dist_env()
    if world > 1:
        print(json.dumps({"workload": args.workload, "unavailable": "single-GPU workload"}))
        return 0
    import torch

    torch.cuda.set_device(local)
    from py4dstem_gb300 import PtychographicTomography, synthetic
    from py4dstem_gb300.tomography import VolumeOps

    tilts = np.linspace(-35.0, 35.0, 8)
    cases = [synthetic.make_scan("tomo", 100 + i, (32, 32), 0.4, 0.05, 64, 160, num_slices=2,
                                 slice_thickness=20.0, backend="torch", device=f"cuda:{local}")
             for i in range(len(tilts))]
    p = PtychographicTomography(
        energy=300e3, num_slices=8, tilt_orientation_matrices=[tilt_matrix(a) for a in tilts],
        datacube=[c.datacube for c in cases], semiangle_cutoff=20.0, defocus=100.0,
        initial_scan_positions=[c.scan_positions_ang for c in cases],
        object_padding_px=(16, 16), verbose=False, device="gpu")
    p.preprocess(plot_probe_overlaps=False, diffraction_patterns_rotate_degrees=0.0,
                 diffraction_patterns_transpose=False)
    J = int(p._num_diffraction_patterns)
    kw = dict(max_batch_size=256, seed_random=0, progress_bar=False, reset=True)
    p.reconstruct(num_iter=max(args.warmup, 2), **kw)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        ev0.record()
        p.reconstruct(num_iter=args.steps, **kw)
        ev1.record()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = int(p._volume_launches + sum(s.launches for s in p._device_states))

    # one float32 volume rotation on its own (load, three prefilter passes, resample)
    shape = tuple(p._object.shape)
    ops = VolumeOps(shape, 8, torch.device("cuda", local))
    vol = torch.rand(shape, dtype=torch.float32, device=f"cuda:{local}")
    out = torch.empty_like(vol)
    for _ in range(3):
        ops.rotate(vol, out, tilt_matrix(20.0), 0)
    reps = 20
    r0 = torch.cuda.Event(enable_timing=True)
    r1 = torch.cuda.Event(enable_timing=True)
    r0.record()
    for _ in range(reps):
        ops.rotate(vol, out, tilt_matrix(20.0), 0)
    r1.record()
    torch.cuda.synchronize()
    rot_ms = r0.elapsed_time(r1) / reps
    line = {
        "metric": "position updates/s (tomography, 8 tilts, 64^2 det)",
        "value": J * args.steps / (ms * 1e-3), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": max(args.warmup, 2), "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "tomography", "tilts": len(tilts), "positions": J,
                   "positions_per_tilt": J // len(tilts), "batch": 256, "slices": 8,
                   "detector": 64, "volume": list(shape), "method": "GD",
                   "collective_measurement_updates": True},
        "volume_rotation_ms": rot_ms,
        "volume_rotation_gvoxels_per_s": float(np.prod(shape)) / (rot_ms * 1e-3) / 1e9,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ learned init
def run_learned_init(args):
    """The learned initializer on the throughput workload's generator: train the
    U-Net on args.li_scans generated 128 x 128 scans (lattice 2.5-5 A, defocus
    0-200 A, 1e5 e-/pattern), then for args.li_seeds held-out scans run the plain
    reconstruction (args.li_iterations iterations of batch 1024) and the learned
    start until it reaches the plain run's final error. value = median over the
    seeds of (learned wall time, network included) / (plain wall time to first
    reach that error); a seed whose learned run never reaches it falls back to
    the plain start and counts as (learned attempt + plain run) / plain run."""
    rank, world, local = dist_env()
    if world > 1:
        print(json.dumps({"workload": "learned-init", "unavailable": "single-GPU workload"}))
        return 0
    import torch

    torch.cuda.set_device(local)
    from py4dstem_gb300 import SingleslicePtychography, learned_init as li, synthetic

    geom = li.ScanGeometry()
    t0 = time.time()
    X, Y = li.generate_training_set(args.li_scans, geom, seed=11)
    torch.cuda.synchronize()
    gen_s = time.time() - t0
    net = li.UNet(seed=0)
    t0 = time.time()
    hist = li.train(net, X, Y, epochs=args.li_epochs, batch=16, lr=1e-3, seed=0)
    torch.cuda.synchronize()
    train_s = time.time() - t0
    target_var = float(Y.var())
    del X, Y
    # convolution FLOPs of one forward pass of a 128 x 128 input (a training
    # step is three such GEMM passes: forward, input and weight gradients)
    conv_flops = 0
    cin = (8, 32, 32, 64, 64, 128, 128, 256, 384, 128, 192, 64, 96, 32)
    cout = (32, 32, 64, 64, 128, 128, 256, 256, 128, 128, 64, 64, 32, 32)
    level = (0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0)
    for ci, co, lv in zip(cin, cout, level):
        conv_flops += 2 * (128 >> lv) ** 2 * 9 * ci * co
    steps = (args.li_scans // 16) * args.li_epochs
    rng = np.random.default_rng(2026)
    results = []
    for k in range(args.li_seeds):
        a = float(rng.uniform(2.5, 5.0))
        df = float(rng.integers(0, 201))
        case = synthetic.make_scan("held-out", 50000 + k, (128, 128), 0.75, 0.05, 128, 512,
                                   dose=1e5, defocus=df, lattice_a=a, backend="torch",
                                   device=f"cuda:{local}")
        p = SingleslicePtychography(datacube=case.datacube, verbose=False, device="gpu",
                                    **case.ctor_kwargs)
        p.preprocess(**case.preprocess_kwargs)
        r = li.compare_starts(net, p, geom, args.li_iterations, 1024, seed=k,
                              true_object=case.true_object)
        pe, le = r.pop("plain_errors"), r.pop("learned_errors")
        po, lo = r.pop("plain_object_errors"), r.pop("learned_object_errors")
        if r["fallback"]:
            r["time_ratio"] = (r["network_s"] + 2.0 * r["plain_s"]) / r["plain_s_to_target"]
        r.update({"lattice_a": a, "defocus": df, "plain_error_curve": pe[::10],
                  "learned_error_curve": le[::10], "plain_object_error_curve": po[::10],
                  "learned_object_error_curve": lo[::10]})
        results.append(r)
        del case, p
    ratios = [r["time_ratio"] for r in results]
    its = [r["learned_iterations"] for r in results if r["learned_iterations"]]
    line = {
        "metric": "time-to-target NMSE, learned vs plain init (learned wall time / plain)",
        "value": float(statistics.median(ratios)), "unit": "ratio", "n_gpus": 1,
        "higher_is_better": False, "steps": args.li_seeds, "warmup": 0, "dtype": "bf16",
        "data": "synthetic",
        "config": {"workload": "learned-init", "train_scans": args.li_scans,
                   "epochs": args.li_epochs, "held_out_seeds": args.li_seeds,
                   "plain_iterations": args.li_iterations, "scan": [128, 128],
                   "detector": 128, "object": [512, 512], "batch": 1024},
        "fallbacks": int(sum(r["fallback"] for r in results)),
        "object_error_time_ratio_median": (float(statistics.median(
            [r["object_time_ratio"] for r in results if r["object_time_ratio"] is not None]))
            if any(r["object_time_ratio"] is not None for r in results) else None),
        "object_error_reached": int(sum(r["learned_object_iterations"] is not None
                                        for r in results)),
        "median_learned_iterations": float(statistics.median(its)) if its else None,
        "median_plain_iterations_to_target": float(statistics.median(
            [r["plain_first_at_target"] for r in results])),
        "generation_s": gen_s, "train_s": train_s, "train_loss": hist,
        "target_variance": target_var,
        "conv_tflops_train": 3 * conv_flops * 16 * steps / train_s / 1e12,
        "seeds": results,
    }
    print(json.dumps(line), flush=True)
    return 0


def main(argv=None):
    args = parse_args(argv)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "multiscan":
        return run_multiscan(args)
    if args.workload == "multislice":
        return run_multislice(args)
    if args.workload in ("projection", "poscorr", "mixed-multislice", "gd256"):
        return run_variant(args)
    if args.workload == "learned-init":
        return run_learned_init(args)
    if args.workload == "tomography":
        return run_tomography(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
