"""Learned initial object for the ptychographic reconstruction.

A 4-level U-Net (32 base channels, BF16 weights and activations, FP32
accumulation) maps a scan's virtual bright-field image and centre-of-mass
magnitude image to the object phase at the scan positions. That phase,
interpolated onto the object grid as exp((-0.1 + i) phase), becomes the
`initial_object_guess` of the reconstruction classes (the reference's entry
point for a start object, singleslice_ptychography.py:118-141). The plain
iterative reconstruction then refines the start and judges it. Where the
learned start ends above the plain run's data error, the plain start is used
instead (:func:`reconstruct_with_fallback`).

Everything runs on the GPU in this library's own kernels: the network
(tensor-core implicit-GEMM convolutions, libptycho_gb300 ``ptycho_nn_*``), its
training data (the ptychographic forward model of the benchmark generator, the
Poisson noise of the virtual-detector sums, ``ptycho_nn_lattice_objects`` /
``ptycho_nn_scan_images``), and
its input at inference (``ptycho_nn_virtual_images`` on the preprocessed
amplitudes). PyTorch only holds device memory.

The reference has no learned component; this module has no reference
counterpart.
"""

from __future__ import annotations

import ctypes
import dataclasses
import math
import time
from typing import Optional, Sequence

import numpy as np

from . import _native
from .optics import ComplexProbe, electron_wavelength_angstrom
from .synthetic import positions_in_pixels, raster_positions


def _torch():
    import torch

    return torch


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check(status: int) -> None:
    if status != 0:
        msg = _native.lib().ptycho_nn_last_error().decode(errors="replace")
        if not msg:
            msg = _native.lib().ptycho_last_error().decode(errors="replace")
        raise _native.PtychoError(status, msg)


@dataclasses.dataclass
class ScanGeometry:
    """The scan and detector of the training generator (the single-slice
    throughput workload): a raster of scan_shape positions at step_ang with
    +-jitter_ang uniform jitter, a detector x detector detector, a square object
    of object_px pixels at sampling_ang, 300 kV and a 20 mrad aperture."""

    scan_shape: tuple = (128, 128)
    step_ang: float = 0.75
    jitter_ang: float = 0.05
    detector: int = 128
    object_px: int = 512
    sampling_ang: float = 0.25
    energy: float = 300e3
    semiangle_mrad: float = 20.0
    dose: float = 1e5
    lattice_range: tuple = (2.5, 5.0)
    defocus_range: tuple = (0.0, 200.0)
    # the target is the object phase blurred to about the probe's resolution
    # (a point sample between scan positions 3 pixels apart would alias the
    # 0.4 A atoms)
    target_blur_ang: float = 0.5

    @property
    def bf_radius_px(self) -> float:
        """The bright-field disc radius in detector pixels."""
        lam = electron_wavelength_angstrom(self.energy)
        dk_mrad = lam * 1e3 / (self.sampling_ang * self.detector)
        return self.semiangle_mrad / dk_mrad


def probe_spectra(geom: ScanGeometry, defoci: Sequence[float]) -> np.ndarray:
    """FFT2 of the probe for each defocus (complex64, (D, det, det))."""
    out = []
    for df in defoci:
        pr = ComplexProbe(energy=geom.energy, gpts=(geom.detector, geom.detector),
                          sampling=(geom.sampling_ang, geom.sampling_ang),
                          semiangle_cutoff=geom.semiangle_mrad, rolloff=2.0,
                          parameters={"defocus": float(df)}).build()._array
        out.append(np.fft.fft2(pr).astype(np.complex64))
    return np.stack(out)


def standardize(img):
    """Per-image zero mean, unit standard deviation (torch, last two axes)."""
    m = img.mean(dim=(-2, -1), keepdim=True)
    s = img.std(dim=(-2, -1), keepdim=True).clamp_min(1e-12)
    return (img - m) / s


def network_input(bf, com_x, com_y):
    """(..., H, W, 2) float32: standardized bright-field and |centre of mass|."""
    torch = _torch()
    com = torch.sqrt(com_x * com_x + com_y * com_y)
    return torch.stack([standardize(bf), standardize(com)], dim=-1).contiguous()


def generate_training_set(num_scans: int, geom: ScanGeometry = ScanGeometry(), seed: int = 0,
                          chunk: int = 32, device: str = "cuda"):
    """Synthetic (input, target) pairs on the GPU. Each scan draws a lattice
    constant, a rotation, an offset, a defocus (whole Angstrom) and its own
    position jitter; returns inputs (num_scans, H, W, 2) and target phases
    (num_scans, H, W) as float32 device tensors."""
    torch = _torch()
    lib = _native.lib()
    dev = torch.device(device)
    rng = np.random.default_rng(seed)
    nx, ny = geom.scan_shape
    J = nx * ny
    P = geom.object_px
    defoci = np.arange(int(geom.defocus_range[0]), int(geom.defocus_range[1]) + 1)
    spectra_all = torch.from_numpy(probe_spectra(geom, defoci)).to(dev)
    inputs = torch.empty((num_scans, nx, ny, 2), dtype=torch.float32, device=dev)
    targets = torch.empty((num_scans, nx, ny), dtype=torch.float32, device=dev)
    stream = _stream()
    for s0 in range(0, num_scans, chunk):
        n = min(chunk, num_scans - s0)
        params = np.zeros((n, 5), np.float32)
        params[:, 0] = rng.uniform(*geom.lattice_range, size=n)
        params[:, 1] = rng.uniform(0.0, np.pi / 2, size=n)
        params[:, 2] = rng.uniform(0.0, 1.0, size=n) * params[:, 0]
        params[:, 3] = rng.uniform(0.0, 1.0, size=n) * params[:, 0]
        dfi = rng.integers(0, len(defoci), size=n)
        pos = np.empty((n, J, 2), np.float32)
        for k in range(n):
            pa = raster_positions(nx, ny, geom.step_ang, geom.jitter_ang, rng)
            pos[k] = positions_in_pixels(pa, geom.sampling_ang, (geom.detector,) * 2, (P, P))
        tparams = torch.from_numpy(params).to(dev)
        tpos = torch.from_numpy(pos).to(dev)
        spectra = spectra_all[torch.from_numpy(dfi).to(dev)].contiguous()
        phase = torch.empty((n, P, P), dtype=torch.float32, device=dev)
        blur = torch.empty_like(phase)
        obj = torch.empty((n, P, P), dtype=torch.complex64, device=dev)
        _check(lib.ptycho_nn_lattice_objects(n, P, geom.sampling_ang, _p(tparams), 0.4, 0.3,
                                             geom.target_blur_ang, _p(phase), _p(blur), _p(obj),
                                             stream))
        bf = torch.empty((n, J), dtype=torch.float32, device=dev)
        cx, cy, tg = torch.empty_like(bf), torch.empty_like(bf), torch.empty_like(bf)
        _check(lib.ptycho_nn_scan_images(n, J, P, _p(spectra), _p(obj), _p(blur), _p(tpos),
                                         geom.dose, geom.bf_radius_px,
                                         seed * 1000003 + s0, _p(bf), _p(cx), _p(cy), _p(tg),
                                         stream))
        shape = (n, nx, ny)
        inputs[s0:s0 + n] = network_input(bf.view(shape), cx.view(shape), cy.view(shape))
        targets[s0:s0 + n] = tg.view(shape)
    return inputs, targets


class UNet:
    """The network's parameters and a per-shape workspace (device memory owned
    here, all computation in libptycho_gb300)."""

    def __init__(self, seed: int = 0, device: str = "cuda"):
        torch = _torch()
        self.lib = _native.lib()
        self.device = torch.device(device)
        nbytes = int(self.lib.ptycho_nn_unet_param_bytes())
        self.params = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        _check(self.lib.ptycho_nn_unet_init(_p(self.params), int(seed), _stream()))
        self._ws = {}
        self.step = 0

    def workspace(self, nb, H, W):
        torch = _torch()
        key = (nb, H, W)
        if key not in self._ws:
            nbytes = int(self.lib.ptycho_nn_unet_workspace_bytes(nb, H, W))
            if nbytes == 0:
                raise ValueError(f"unsupported network input {nb}x{H}x{W} "
                                 "(height and width must be multiples of 64)")
            self._ws[key] = (torch.zeros(nbytes, dtype=torch.uint8, device=self.device), nbytes)
        return self._ws[key]

    def forward(self, inputs):
        """inputs (nb, H, W, 2) float32 device tensor -> (nb, H, W)."""
        torch = _torch()
        nb, H, W, _ = inputs.shape
        ws, nbytes = self.workspace(nb, H, W)
        out = torch.empty((nb, H, W), dtype=torch.float32, device=self.device)
        _check(self.lib.ptycho_nn_unet_forward(_p(self.params), _p(inputs.contiguous()), nb, H,
                                               W, _p(out), _p(ws), nbytes, _stream()))
        return out

    def train_step(self, inputs, targets, lr, loss_out, mask=None):
        nb, H, W, _ = inputs.shape
        ws, nbytes = self.workspace(nb, H, W)
        self.step += 1
        count = float(nb * H * W) if mask is None else float(mask.sum().item())
        _check(self.lib.ptycho_nn_unet_train_step(
            _p(self.params), _p(inputs), _p(targets), _p(mask), count, nb, H, W, float(lr),
            self.step, _p(loss_out), _p(ws), nbytes, _stream()))

    def check(self):
        for (nb, H, W), (ws, _) in self._ws.items():
            _check(self.lib.ptycho_nn_check(_p(ws), nb, H, W, _stream()))

    def state_bytes(self) -> np.ndarray:
        return self.params.cpu().numpy()

    def load_state_bytes(self, data: np.ndarray) -> None:
        torch = _torch()
        self.params.copy_(torch.from_numpy(np.ascontiguousarray(data, dtype=np.uint8)))


def train(net: UNet, inputs, targets, epochs: int = 8, batch: int = 16, lr: float = 1e-3,
          seed: int = 0, log=None):
    """Adam over shuffled mini-batches with a cosine learning-rate decay; returns
    the mean loss of each epoch (one device-to-host read per epoch)."""
    torch = _torch()
    n = inputs.shape[0]
    steps_per_epoch = n // batch
    total = steps_per_epoch * epochs
    rng = np.random.default_rng(seed)
    loss = torch.zeros(steps_per_epoch, dtype=torch.float32, device=inputs.device)
    history = []
    k = 0
    for ep in range(epochs):
        order = torch.from_numpy(rng.permutation(n)).to(inputs.device)
        for b in range(steps_per_epoch):
            idx = order[b * batch:(b + 1) * batch]
            xb = inputs[idx].contiguous()
            yb = targets[idx].contiguous()
            rate = lr * 0.5 * (1.0 + math.cos(math.pi * k / max(1, total)))
            net.train_step(xb, yb, rate, loss[b:b + 1])
            k += 1
        net.check()
        history.append(float(loss.mean().item()))
        if log:
            log(f"epoch {ep + 1}/{epochs}: loss {history[-1]:.5f}")
    return history


# ------------------------------------------------------------------ inference
def scan_images(ptycho, geom: ScanGeometry):
    """Virtual bright-field and centre-of-mass images of a preprocessed
    reconstruction object (its amplitudes, corner-centred), as (H, W) tensors on
    the scan grid."""
    torch = _torch()
    lib = _native.lib()
    amps = ptycho._amplitudes
    if not isinstance(amps, torch.Tensor):
        amps = torch.from_numpy(np.ascontiguousarray(amps, dtype=np.float32))
    amps = amps.to(device="cuda", dtype=torch.float32).contiguous()
    J, sx, sy = amps.shape
    bf = torch.empty(J, dtype=torch.float32, device="cuda")
    cx, cy = torch.empty_like(bf), torch.empty_like(bf)
    _check(lib.ptycho_nn_virtual_images(_p(amps), J, sx, sy, geom.bf_radius_px, _p(bf), _p(cx),
                                        _p(cy), _stream()))
    shape = tuple(int(v) for v in ptycho._datacube.Rshape) if hasattr(ptycho, "_datacube") \
        and ptycho._datacube is not None else None
    if shape is None or shape[0] * shape[1] != J:
        n = int(round(math.sqrt(J)))
        shape = (n, n)
    return bf.view(shape), cx.view(shape), cy.view(shape)


def _pad64(x):
    """Pad the last two axes of (H, W) images up to multiples of 64 (edge values)."""
    torch = _torch()
    H, W = x.shape[-2:]
    Hp, Wp = -(-H // 64) * 64, -(-W // 64) * 64
    if (Hp, Wp) == (H, W):
        return x
    return torch.nn.functional.pad(x[None], (0, Wp - W, 0, Hp - H), mode="replicate")[0]


def predict_phase(net: UNet, ptycho, geom: ScanGeometry = ScanGeometry()):
    """The network's phase at the scan positions of a preprocessed object (H, W)."""
    bf, cx, cy = scan_images(ptycho, geom)
    H, W = bf.shape
    x = network_input(_pad64(bf), _pad64(cx), _pad64(cy))[None]
    return net.forward(x)[0, :H, :W]


def phase_to_object(phase_grid: np.ndarray, positions_px: np.ndarray, object_shape,
                    scan_shape) -> np.ndarray:
    """exp((-0.1 + i) phase) on the object grid: the scan-grid phase is placed by
    an affine fit of the positions to the scan indices and interpolated
    bilinearly; outside the scanned area the phase is zero."""
    nx, ny = scan_shape
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    A = np.stack([ix.ravel(), iy.ravel(), np.ones(nx * ny)], axis=1)
    coef, *_ = np.linalg.lstsq(A, positions_px.astype(np.float64), rcond=None)
    M = coef[:2].T  # pixel = M (ix, iy) + t
    t = coef[2]
    Minv = np.linalg.inv(M)
    Px, Py = object_shape
    gx, gy = np.meshgrid(np.arange(Px), np.arange(Py), indexing="ij")
    uv = np.stack([gx.ravel() - t[0], gy.ravel() - t[1]], axis=0)
    u, v = (Minv @ uv)
    inside = (u >= 0) & (u <= nx - 1) & (v >= 0) & (v <= ny - 1)
    u = np.clip(u, 0, nx - 1)
    v = np.clip(v, 0, ny - 1)
    u0 = np.minimum(np.floor(u).astype(int), nx - 2)
    v0 = np.minimum(np.floor(v).astype(int), ny - 2)
    fu, fv = u - u0, v - v0
    g = phase_grid
    ph = ((1 - fu) * (1 - fv) * g[u0, v0] + fu * (1 - fv) * g[u0 + 1, v0] +
          (1 - fu) * fv * g[u0, v0 + 1] + fu * fv * g[u0 + 1, v0 + 1])
    ph = np.where(inside, ph, 0.0).reshape(Px, Py)
    return np.exp((-0.1 + 1j) * ph).astype(np.complex64)


def initial_object(net: UNet, ptycho, geom: ScanGeometry = ScanGeometry()) -> np.ndarray:
    """The learned start object for a preprocessed single-slice reconstruction."""
    phase = predict_phase(net, ptycho, geom).cpu().numpy()
    return phase_to_object(phase, np.asarray(ptycho._positions_px), np.shape(ptycho._object),
                           phase.shape)


@dataclasses.dataclass
class TimeToTarget:
    """Iterations and wall time for a run to reach a data error."""

    iterations: Optional[int]
    seconds: Optional[float]
    errors: list


def iterations_to_target(errors: Sequence[float], target: float) -> Optional[int]:
    for k, e in enumerate(errors):
        if e <= target:
            return k + 1
    return None


def reconstruct_with_fallback(make_ptycho, net: UNet, num_iter: int, geom: ScanGeometry,
                              reconstruct_kwargs: dict, target_error: float):
    """The learned start, refined by the plain reconstruction for at most
    num_iter iterations, stopping at the first iteration whose error is at or
    below target_error. Returns (ptycho, iterations or None, seconds, used
    learned start). When the learned run does not reach the target, the plain
    start is used instead (the fallback) and the learned result discarded."""
    torch = _torch()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    p = make_ptycho(None)
    guess = initial_object(net, p, geom)
    p = make_ptycho(guess)
    errs = []
    for _ in range(num_iter):
        p.reconstruct(num_iter=1, **reconstruct_kwargs)
        errs.append(float(p.error))
        if errs[-1] <= target_error:
            break
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    k = iterations_to_target(errs, target_error)
    if k is not None:
        return p, k, dt, True
    q = make_ptycho(None)
    q.reconstruct(num_iter=num_iter, **reconstruct_kwargs)
    return q, None, dt, False


def object_nmse(obj, true_obj, mask):
    """min over a complex scalar c of sum_mask |O - c T|^2 / sum_mask |T|^2 (the
    object error up to the global phase and scale the data do not fix); torch
    tensors on the device, mask boolean."""
    o = obj[mask].to(_torch().complex128)
    t = true_obj[mask].to(_torch().complex128)
    tt = (t.conj() * t).real.sum()
    c = (t.conj() * o).sum() / tt
    r = o - c * t
    return float(((r.conj() * r).real.sum() / tt).item())


def run_to_target(ptycho, object_init, max_iter: int, target: Optional[float], batch: int,
                  seed: int, step_size: float = 0.5, true_object=None):
    """Gradient-descent iterations of a preprocessed single-slice object from
    `object_init` (None: its own initial object) through the device state and
    the graph-replayed iteration driver of reconstruct(), reading the error
    after every iteration like the reference; stops after max_iter iterations or
    at the first error <= target. Returns the errors and, for each iteration,
    the seconds since the start (state set-up included). With `true_object`
    (the object on the reconstruction grid) the object error (object_nmse over
    the field-of-view mask) after each iteration is returned too; its
    evaluation is not counted in the times."""
    torch = _torch()
    from . import engine

    p = ptycho
    J = p._num_diffraction_patterns
    B = min(batch, J)
    obj = np.asarray(p._object) if object_init is None else object_init
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = engine.create_state(
        roi_shape=tuple(p._region_of_interest_shape), object_array=np.asarray(obj),
        probe_array=p._probe, amplitudes=p._amplitudes_for_state(), positions_px=p._positions_px,
        num_slices=1, num_probes=1, potential=False, max_batch=B, storage="gpu",
        fov_mask_inverse=p._object_fov_mask_inverse)
    drv = engine.IterationDriver(st, graph=True, max_batch=B, step_size=step_size,
                                 normalization_min=1.0,
                                 use_mask=bool(p._object_fov_mask_inverse.sum() > 0),
                                 mean_intensity=p._mean_diffraction_intensity)
    rs = np.random.RandomState(seed)
    order = np.arange(J)
    errors, times, obj_err = [], [], []
    if true_object is not None:
        tobj = torch.from_numpy(np.asarray(true_object, dtype=np.complex64)).to(st.object.device)
        mask = torch.from_numpy(np.asarray(p._object_fov_mask, dtype=bool)).to(st.object.device)
    excluded = 0.0
    for _ in range(max_iter):
        rs.shuffle(order)
        drv.iterate(order)
        errors.append(float(drv.error()))  # synchronises
        times.append(time.perf_counter() - t0 - excluded)
        if true_object is not None:
            t1 = time.perf_counter()
            obj_err.append(object_nmse(st.object.view(tobj.shape), tobj, mask))
            excluded += time.perf_counter() - t1
        if target is not None and errors[-1] <= target:
            break
    if true_object is not None:
        return errors, times, obj_err
    return errors, times


def compare_starts(net: UNet, ptycho, geom: ScanGeometry, plain_iter: int, batch: int,
                   seed: int, true_object=None):
    """The plain start run for plain_iter iterations, then the learned start run
    until it reaches the plain run's final data error (at most plain_iter
    iterations). Times compare the first iteration at which each run reaches
    that error; the learned run's time includes the network input, the network
    and the start object. Returns a dict; `fallback` is True when the learned
    run did not reach the target (the plain result then stands). With
    `true_object`, both runs also record the object error after each iteration
    and the dict gives the iterations each needs to reach the plain run's final
    object error (both runs then go the full plain_iter iterations)."""
    torch = _torch()
    track = true_object is not None
    out = run_to_target(ptycho, None, plain_iter, None, batch, seed, true_object=true_object)
    plain, t_plain = out[0], out[1]
    target = plain[-1]
    # the plain run reaches its final error first at iteration kp (its error
    # need not fall monotonically)
    kp = iterations_to_target(plain, target)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    guess = initial_object(net, ptycho, geom)
    torch.cuda.synchronize()
    t_net = time.perf_counter() - t0
    out_l = run_to_target(ptycho, guess, plain_iter, None if track else target, batch, seed,
                          true_object=true_object)
    learned, t_learned = out_l[0], out_l[1]
    k = iterations_to_target(learned, target)
    t_l = t_net + t_learned[k - 1] if k is not None else None
    res = {"plain_iterations": plain_iter, "plain_error": target,
           "plain_first_at_target": kp, "plain_s_to_target": t_plain[kp - 1],
           "plain_s": t_plain[-1], "learned_iterations": k, "learned_s": t_l,
           "network_s": t_net, "learned_first_error": learned[0],
           "plain_first_error": plain[0], "fallback": k is None,
           "time_ratio": t_l / t_plain[kp - 1] if k is not None else None,
           "plain_errors": plain, "learned_errors": learned[:k] if k else learned}
    if track:
        po, lo = out[2], out_l[2]
        ot = po[-1]
        kpo = iterations_to_target(po, ot)
        klo = iterations_to_target(lo, ot)
        res.update({"plain_object_error": ot, "learned_start_object_error": lo[0],
                    "plain_start_object_error": po[0],
                    "plain_object_first_at_target": kpo, "learned_object_iterations": klo,
                    "object_time_ratio": ((t_net + t_learned[klo - 1]) / t_plain[kpo - 1]
                                          if klo is not None else None),
                    "plain_object_errors": po, "learned_object_errors": lo})
    return res
