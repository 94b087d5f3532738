"""Many independent scans reconstructed together on one GPU.

``MultiScanReconstruction`` takes preprocessed drop-in instances
(``SingleslicePtychography``, ``MultislicePtychography``,
``MixedstatePtychography``; any mix of scan grids and detector sizes) and runs
gradient-descent iterations on all of them at once:

* every scan keeps its own device state (object, probe, resident amplitudes,
  workspace) and its own CUDA stream, so the batches of small scans, which do
  not fill the GPU alone, run concurrently with those of the others;
* one iteration of all scans (every batch, the per-iteration constraints, the
  mixed-state orthogonalisation on the device) is captured once as a CUDA graph
  and replayed, so an iteration is one graph launch plus two small copies (the
  next position orders in, the per-scan errors out), with no host round trip;
* the launch configuration (scans on concurrent streams or one after another,
  and, when asked, the batch size) is chosen by timing the candidates on a
  snapshot of the state (``py4dstem_gb300.autotune``), once per configuration.

Each scan follows the reference's loop (singleslice_ptychography.py:836-996 and
its multislice / mixed-state twins) with its own random stream: scan k shuffles
its positions with ``numpy.random.RandomState(seed_random + k)``, so it sees the
same position orders as a single reconstruction of that scan after
``np.random.seed(seed_random + k)``. Mixed-state modes are orthogonalised on the
device (phase convention of ``ptycho_probe_orthogonalize``).
"""

from __future__ import annotations

import ctypes
from typing import List, Sequence, Union

import numpy as np

from . import _native, autotune, engine


class MultiScanReconstruction:
    def __init__(self, ptychographies: Sequence, *,
                 max_batch_size: Union[int, str, Sequence[int], None] = 256,
                 seed_random: int = 0, step_size: float = 0.5, normalization_min: float = 1.0,
                 fix_probe: bool = False, fix_probe_com: bool = True,
                 orthogonalize_probe: bool = True, shrinkage_rad: float = 0.0,
                 fix_potential_baseline: bool = True, pure_phase_object: bool = False,
                 object_positivity: bool = True, use_graph: bool = True,
                 concurrent: Union[bool, str] = "auto"):
        if not ptychographies:
            raise ValueError("no scans given")
        for p in ptychographies:
            if not getattr(p, "_preprocessed", False):
                raise ValueError("every scan must be preprocessed first")
        self.scans = list(ptychographies)
        n = len(self.scans)
        self.tune_batch = isinstance(max_batch_size, str)
        if self.tune_batch and max_batch_size != "auto":
            raise ValueError("max_batch_size must be an int, a list of ints or 'auto'")
        if isinstance(max_batch_size, (list, tuple)):
            if len(max_batch_size) != n:
                raise ValueError("one max_batch_size per scan")
            self.batch = [int(b) for b in max_batch_size]
        elif max_batch_size is None:
            self.batch = [p._num_diffraction_patterns for p in self.scans]
        elif self.tune_batch:
            self.batch = [min(256, p._num_diffraction_patterns) for p in self.scans]
        else:
            self.batch = [int(max_batch_size)] * n
        self.seed = int(seed_random)
        self.options = dict(step_size=step_size, normalization_min=normalization_min,
                            fix_probe=fix_probe, fix_probe_com=fix_probe_com,
                            orthogonalize_probe=orthogonalize_probe,
                            shrinkage_rad=shrinkage_rad, pure_phase=pure_phase_object,
                            positivity=object_positivity)
        self.fix_potential_baseline = fix_potential_baseline
        self.use_graph = bool(use_graph)
        self.concurrent = concurrent
        self.tuning = None
        self._built = False

    # ------------------------------------------------------------------ setup
    def _build(self):
        torch = engine._torch()
        dev = torch.device("cuda", torch.cuda.current_device())
        self.torch = torch
        n = len(self.scans)
        self.J = [p._num_diffraction_patterns for p in self.scans]
        jmax = max(self.J)
        self.order_all = torch.zeros((n, jmax), dtype=torch.int32, device=dev)
        self.acc_all = torch.zeros(n, dtype=torch.float32, device=dev)
        self.states, self.drivers = [], []
        for k, p in enumerate(self.scans):
            st, drv = self._make_state(k, p, self.batch[k])
            self.states.append(st)
            self.drivers.append(drv)
        self.streams = [torch.cuda.Stream() for _ in range(n)]
        self.root = torch.cuda.Stream()
        lib = _native.lib()
        for s in self.streams + [self.root]:
            _native.check(lib.ptycho_prepare_stream(ctypes.c_void_p(s.cuda_stream)))
        self.rngs = [np.random.RandomState(self.seed + k) for k in range(n)]
        self.shuffled = [np.arange(j) for j in self.J]
        self._graphs = {}
        self._built = True

    def _make_state(self, k, p, batch):
        potential = p._object_type == "potential"
        obj = np.asarray(p._object, dtype=np.float32 if potential else np.complex64)
        use_mask = bool(self.fix_potential_baseline and p._object_fov_mask_inverse.sum() > 0)
        st = engine.create_state(
            roi_shape=tuple(p._region_of_interest_shape), object_array=obj,
            probe_array=p._probe, amplitudes=p._amplitudes, positions_px=p._positions_px,
            num_slices=p._num_slices, num_probes=p._num_probes, potential=potential,
            max_batch=int(batch), storage="gpu",
            propagators=getattr(p, "_propagator_arrays", None) if p._multislice else None,
            fov_mask_inverse=p._object_fov_mask_inverse if use_mask else None,
            mixed_state=p._mixed)
        # error accumulator and order row are views into the shared per-scan arrays
        st.error_accum = self.acc_all[k:k + 1]
        st.order = self.order_all[k, :self.J[k]]
        o = self.options
        drv = engine.IterationDriver(
            st, max_batch=int(batch), step_size=o["step_size"],
            normalization_min=o["normalization_min"], fix_probe=o["fix_probe"],
            shrinkage_rad=o["shrinkage_rad"], use_mask=use_mask,
            pure_phase=o["pure_phase"] and not potential, positivity=o["positivity"],
            fix_probe_com=o["fix_probe_com"], orthogonalize_probe=o["orthogonalize_probe"],
            mean_intensity=p._mean_diffraction_intensity, device_orthogonalization=True)
        return st, drv

    # -------------------------------------------------------------- one iteration
    def _issue(self, concurrent: bool):
        """Issue one iteration of every scan on the current (root) stream."""
        torch = self.torch
        root = torch.cuda.current_stream()
        if not concurrent:
            for drv in self.drivers:
                drv.iterate(None)
            return
        for s in self.streams:
            s.wait_stream(root)
        for drv, s in zip(self.drivers, self.streams):
            with torch.cuda.stream(s):
                drv.iterate(None)
        for s in self.streams:
            root.wait_stream(s)

    def _graph(self, concurrent: bool):
        # a captured graph holds the kernels chosen at capture time, so it is
        # kept per 128^2 kernel schedule as well
        key = (concurrent, _native.lib().ptycho_set_kernel_schedule(128, 0))
        _native.lib().ptycho_set_kernel_schedule(128, key[1])
        if key not in self._graphs:
            torch = self.torch
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=self.root):
                self._issue(concurrent)
            self._graphs[key] = g
        return self._graphs[key]

    def _next_orders(self):
        rows = np.zeros(tuple(self.order_all.shape), dtype=np.int32)
        for k, (rng, sh) in enumerate(zip(self.rngs, self.shuffled)):
            rng.shuffle(sh)
            rows[k, :self.J[k]] = sh
        return rows

    def _run_iteration(self, concurrent: bool, orders_dev, it):
        self.order_all.copy_(orders_dev[it])
        if self.use_graph:
            self._graph(concurrent).replay()
        else:
            self._issue(concurrent)

    # ------------------------------------------------------------------ tuning
    def _snapshot(self):
        return [(st.object.clone(), st.probe.clone()) for st in self.states]

    def _restore(self, snap):
        for st, (o, p) in zip(self.states, snap):
            st.object.copy_(o)
            st.probe.copy_(p)

    def _tune(self, orders_dev):
        """Scans on concurrent streams or one after another: one iteration of each,
        timed on a snapshot of the state that is restored afterwards."""
        torch = self.torch
        key = ("multiscan", self.use_graph, tuple(self.J), tuple(self.batch),
               tuple(tuple(p._region_of_interest_shape) for p in self.scans),
               tuple((p._num_slices, p._num_probes) for p in self.scans))
        concs = [True, False] if self.concurrent == "auto" else [bool(self.concurrent)]
        # the 128 x 128 kernel schedule (1: shared-memory transforms by the whole
        # block, 2: register-resident four-step transforms for single-slice
        # single-probe scans, 3: shared-memory transforms by groups of warps)
        # matters for scans at a 128^2 detector
        eligible = any(tuple(p._region_of_interest_shape) == (128, 128) for p in self.scans)
        scheds = [1, 2, 3] if eligible else [0]
        cands = [{"concurrent": c, "schedule": sc} for c in concs for sc in scheds]
        key = key + (tuple((c["concurrent"], c["schedule"]) for c in cands),)
        lib = _native.lib()

        def run(c):
            prev = lib.ptycho_set_kernel_schedule(128, c["schedule"])
            try:
                self._run_iteration(c["concurrent"], orders_dev, 0)
            finally:
                lib.ptycho_set_kernel_schedule(128, prev)

        torch.cuda.synchronize()  # the snapshot must see the finished iteration
        snap = self._snapshot()
        torch.cuda.synchronize()
        with torch.cuda.stream(self.root):
            best, timings = autotune.tune(key, cands, run, warmup=1, reps=3,
                                          device=autotune.device_key())
        torch.cuda.synchronize()
        self._restore(snap)
        torch.cuda.synchronize()  # later iterations run on other streams
        self.tuning = dict(self.tuning or {}, choice=best, timings_ms=timings)
        return best

    def _tune_batch(self, orders_dev):
        """Batch size among 128 / 256 / 512 / 1024 (capped at each scan's size) by
        the time of one concurrent, eager iteration from the initial state; the
        state is rebuilt from the scans' host arrays for every candidate."""
        torch = self.torch
        key = ("multiscan-batch", tuple(self.J),
               tuple(tuple(p._region_of_interest_shape) for p in self.scans),
               tuple((p._num_slices, p._num_probes) for p in self.scans))
        dev = autotune.device_key()
        hit = autotune.lookup(key, dev)
        if hit is not None:
            b_best = hit[0]["batch"]
            self._rebuild([min(b_best, j) for j in self.J])
            torch.cuda.synchronize()
            self.tuning = dict(self.tuning or {}, batch=b_best, batch_timings_ms=hit[1])
            return
        timings = []
        for b in (128, 256, 512, 1024):
            self._rebuild([min(b, j) for j in self.J])
            with torch.cuda.stream(self.root):
                t = autotune.time_candidates(
                    [{"batch": b}], lambda c: (self.order_all.copy_(orders_dev[0]),
                                               self._issue(True)),
                    warmup=1, reps=2)[0][1]
            timings.append(({"batch": b}, t))
        torch.cuda.synchronize()
        b_best = min(timings, key=lambda x: x[1])[0]["batch"]
        autotune.remember(key, {"batch": b_best}, timings, dev)
        self._rebuild([min(b_best, j) for j in self.J])
        torch.cuda.synchronize()
        self.tuning = dict(self.tuning or {}, batch=b_best, batch_timings_ms=timings)

    def _rebuild(self, batch):
        self.batch = list(batch)
        self.states, self.drivers = [], []
        for k, p in enumerate(self.scans):
            st, drv = self._make_state(k, p, self.batch[k])
            self.states.append(st)
            self.drivers.append(drv)
        self._graphs = {}

    # ------------------------------------------------------------------- run
    def reconstruct(self, num_iter: int = 8):
        """Run `num_iter` iterations on every scan; sets each scan's object, probe,
        error and error_iterations like its own reconstruct() would."""
        torch = engine._torch()
        if not self._built:
            self._build()
        n = len(self.scans)
        orders = np.stack([self._next_orders() for _ in range(num_iter)])
        orders_dev = torch.from_numpy(orders).to(self.order_all.device)
        errs = torch.zeros((num_iter, n), dtype=torch.float32, device=self.order_all.device)
        torch.cuda.synchronize()
        if self.tune_batch and "batch" not in (self.tuning or {}):
            self._tune_batch(orders_dev)  # from the initial state, before iteration 0
        with torch.cuda.stream(self.root):
            # the first iteration runs eagerly: it sets up the library's per-stream
            # state, which a graph capture must not do
            self.order_all.copy_(orders_dev[0])
            self._issue(True)
            errs[0].copy_(self.acc_all)
        if "choice" not in (self.tuning or {}) and num_iter > 1:
            best = self._tune(orders_dev)
        else:
            best = (self.tuning or {}).get("choice",
                                           {"concurrent": self.concurrent is not False})
        concurrent = bool(best["concurrent"])
        lib = _native.lib()
        prev = lib.ptycho_set_kernel_schedule(128, int(best.get("schedule", 0)))
        try:
            with torch.cuda.stream(self.root):
                for it in range(1, num_iter):
                    self._run_iteration(concurrent, orders_dev, it)
                    errs[it].copy_(self.acc_all)
        finally:
            lib.ptycho_set_kernel_schedule(128, prev)
        torch.cuda.synchronize()
        self._finish(errs.cpu().numpy())
        return self

    def _finish(self, errs: np.ndarray):
        for k, (p, st) in enumerate(zip(self.scans, self.states)):
            norm = np.float32(p._mean_diffraction_intensity) * self.J[k]
            e = (errs[:, k] / norm).astype(np.float32)
            if getattr(p, "error_iterations", None) is None:
                p.error_iterations = []
            p.error_iterations.extend(float(v) for v in e)
            p.error = float(e[-1])
            p._object = st.object.cpu().numpy()
            p._probe = st.probe.cpu().numpy().reshape(np.shape(p._probe))
            p.object = p._object.copy()
            p.probe = p.probe_centered
            p._exit_waves = None


def reconstruct_many(ptychographies: Sequence, num_iter: int = 8, **kwargs) -> List:
    """Functional form: build a MultiScanReconstruction and run it."""
    MultiScanReconstruction(ptychographies, **kwargs).reconstruct(num_iter)
    return list(ptychographies)
