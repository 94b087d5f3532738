"""The ptychographic forward model as a ``torch.autograd.Function``.

``PtychoForwardModel.loss(object, probe)`` returns the data error of a set of
scan positions,

    loss = sum_b sum_k (A_bk - |F_bk|)^2,   F_b = FFT2(exit wave of position b),

the batch error of the reference's gradient-descent Fourier projection
(py4DSTEM/process/phase/ptychographic_methods.py:1576-1635, 2742-2804), for
single-slice, multislice and mixed-state models. Its backward is the library's
hand-written adjoint: ``ptycho_gd_gradient`` runs the fused forward + adjoint
position kernel and the deterministic reductions and returns
d loss / d Re + i d loss / d Im for the object (d loss / dV for potentials) and
the probe, which is -2N times the summed adjoint terms of
``_gradient_descent_adjoint`` (ptychographic_methods.py:1818-1908, 2353-2458,
2906-3000) before their normalisation.

Memory. The forward pass runs the forward-only kernel and keeps nothing per
position or per slice; the backward pass recomputes each batch of positions
(forward through every slice, then the adjoint) inside the kernel, with the
per-slice transmitted probes of one batch in the workspace (T x B x N x 12 bytes,
reused batch after batch). Memory therefore scales with the batch size, not with
the number of positions: a 16-slice model at a 128^2 detector needs 3.2 GB of
workspace at B = 1024 and 0.8 GB at B = 256, whatever the scan size.

The kernels run on the current CUDA stream; there is no CPU path.
"""

from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _native
from .preprocess import generate_batches


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("py4dstem_gb300.autograd needs a CUDA GPU (there is no CPU fallback)")
    return torch


def _vp(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class PtychoForwardModel:
    """Data, geometry and workspace of a forward model; `loss` is differentiable.

    amplitudes   (J, Ax, Ay) float32, corner-centred (as preprocess() leaves them)
    positions_px (J, 2) float32 probe positions in object pixels
    object_shape (Px, Py) of one slice
    roi_shape    (Sx, Sy) of the probe and the object patches when it differs from
                 the detector (Ax, Ay): the far field is then resampled between
                 the two grids (region_of_interest_shape); default the detector's
    """

    def __init__(self, amplitudes, positions_px, object_shape, *, num_slices: int = 1,
                 num_probes: int = 1, potential: bool = False, propagators=None,
                 mixed_state: bool = False, max_batch: int = 1024, device=None,
                 roi_shape=None):
        torch = _torch()
        self.torch = torch
        dev = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self.device = dev
        amps = torch.as_tensor(np.ascontiguousarray(amplitudes, dtype=np.float32)
                               if isinstance(amplitudes, np.ndarray) else amplitudes)
        self.amplitudes = amps.to(dev, torch.float32).contiguous()
        pos = torch.as_tensor(np.ascontiguousarray(positions_px, dtype=np.float32)
                              if isinstance(positions_px, np.ndarray) else positions_px)
        self.positions = pos.to(dev, torch.float32).contiguous()
        J, ax, ay = self.amplitudes.shape
        sx, sy = (ax, ay) if roi_shape is None else (int(roi_shape[0]), int(roi_shape[1]))
        self.num_positions = int(J)
        self.roi_shape = (int(sx), int(sy))
        self.num_slices = int(num_slices)
        self.num_probes = int(num_probes)
        self.potential = bool(potential)
        flags = _native.FLAG_MIXED_STATE if (mixed_state or num_probes > 1) else 0
        self.geometry = _native.Geometry(int(sx), int(sy), int(object_shape[-2]),
                                         int(object_shape[-1]), self.num_slices,
                                         self.num_probes, 1 if potential else 0, flags)
        if (ax, ay) != (sx, sy):
            self.geometry.detector_x, self.geometry.detector_y = int(ax), int(ay)
        lib = _native.lib()
        if not lib.ptycho_roi_supported(int(sx), int(sy)):
            raise NotImplementedError(f"no GPU kernel for a {sx}x{sy} region of interest")
        if lib.ptycho_geometry_supported(ctypes.byref(self.geometry)) != _native.PTYCHO_OK:
            raise NotImplementedError(lib.ptycho_last_error().decode())
        self.max_batch = int(min(max_batch, J))
        self.ws_bytes = int(lib.ptycho_workspace_bytes(ctypes.byref(self.geometry),
                                                       self.max_batch))
        self.workspace = torch.empty(self.ws_bytes + 256, dtype=torch.uint8, device=dev)
        self.propagators = None
        if self.num_slices > 1:
            if propagators is None:
                raise ValueError("multislice needs the (T-1, Sx, Sy) propagators")
            self.propagators = torch.as_tensor(
                np.ascontiguousarray(propagators, dtype=np.complex64)).to(dev)
        self.rows = torch.arange(J, dtype=torch.int32, device=dev)
        self._errors = torch.empty(J, dtype=torch.float32, device=dev)
        self._loss = torch.empty(1, dtype=torch.float32, device=dev)

    @classmethod
    def from_ptychography(cls, p, max_batch: int = 1024):
        """Forward model of a preprocessed drop-in class instance."""
        return cls(p._amplitudes, p._positions_px, np.shape(p._object)[-2:],
                   num_slices=p._num_slices, num_probes=p._num_probes,
                   potential=p._object_type == "potential",
                   propagators=getattr(p, "_propagator_arrays", None) if p._multislice else None,
                   mixed_state=p._mixed, max_batch=max_batch,
                   roi_shape=tuple(p._region_of_interest_shape))

    # ------------------------------------------------------------------ helpers
    def _ws(self):
        return ctypes.c_void_p((self.workspace.data_ptr() + 255) & ~255)

    def _stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def _check_inputs(self, obj, probe):
        torch = self.torch
        want_obj = torch.float32 if self.potential else torch.complex64
        if obj.dtype != want_obj or obj.device != self.device:
            raise TypeError(f"object must be {want_obj} on {self.device}")
        if probe.dtype != torch.complex64 or probe.device != self.device:
            raise TypeError(f"probe must be complex64 on {self.device}")
        n_obj = self.num_slices * self.geometry.object_x * self.geometry.object_y
        n_probe = self.num_probes * self.roi_shape[0] * self.roi_shape[1]
        if obj.numel() != n_obj or probe.numel() != n_probe:
            raise ValueError("object / probe sizes do not match the model geometry")
        return obj.contiguous(), probe.contiguous()

    def _chunks(self, rows):
        rows = self.rows if rows is None else rows
        n = int(rows.shape[0])
        for start, end in generate_batches(n, self.max_batch):
            yield rows, start, end

    # ------------------------------------------------------------ kernels
    def position_errors(self, obj, probe, rows=None):
        """Per-position sum_k (A - |F|)^2 (forward-only kernel), float32 (len(rows),)."""
        obj, probe = self._check_inputs(obj, probe)
        lib = _native.lib()
        rows = self.rows if rows is None else rows.to(self.device, self.torch.int32).contiguous()
        out = self.torch.empty(int(rows.shape[0]), dtype=self.torch.float32, device=self.device)
        for r, start, end in self._chunks(rows):
            rp = ctypes.c_void_p(r.data_ptr() + 4 * start)
            _native.check(lib.ptycho_self_consistency_errors(
                ctypes.byref(self.geometry), _vp(obj), _vp(probe), _vp(self.amplitudes), rp,
                _vp(self.positions), rp, end - start, _vp(self.propagators),
                ctypes.c_void_p(out.data_ptr() + 4 * start), self._ws(), self.ws_bytes,
                self._stream()))
        return out

    def loss_and_gradient(self, obj, probe, rows=None, probe_gradient: bool = True):
        """(loss, object gradient, probe gradient) without autograd: the fused
        forward + adjoint kernel, batch by batch, gradients summed over batches."""
        torch = self.torch
        obj, probe = self._check_inputs(obj, probe)
        lib = _native.lib()
        rows = self.rows if rows is None else rows.to(self.device, torch.int32).contiguous()
        g_obj = torch.zeros_like(obj)
        g_probe = torch.zeros_like(probe) if probe_gradient else None
        part_obj = torch.empty_like(obj)
        part_probe = torch.empty_like(probe) if probe_gradient else None
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        for r, start, end in self._chunks(rows):
            rp = ctypes.c_void_p(r.data_ptr() + 4 * start)
            _native.check(lib.ptycho_gd_gradient(
                ctypes.byref(self.geometry), _vp(obj), _vp(probe), _vp(self.amplitudes), rp,
                _vp(self.positions), rp, end - start, None, _vp(self.propagators),
                _vp(part_obj), _vp(part_probe), _vp(self._loss), self._ws(), self.ws_bytes,
                self._stream()))
            g_obj += part_obj
            if probe_gradient:
                g_probe += part_probe
            loss += self._loss
        return loss[0], g_obj, g_probe

    def loss(self, obj, probe, rows=None):
        """Differentiable data error of the positions `rows` (all when None)."""
        return _ForwardLoss.apply(obj, probe, self, rows)


class _ForwardLoss:
    """Created lazily so that importing this module does not import torch."""

    _cls = None

    @classmethod
    def apply(cls, obj, probe, model, rows):
        if cls._cls is None:
            torch = _torch()

            class ForwardLoss(torch.autograd.Function):
                @staticmethod
                def forward(ctx, obj_, probe_, model_, rows_):
                    ctx.model = model_
                    ctx.rows = rows_
                    ctx.save_for_backward(obj_, probe_)
                    errors = model_.position_errors(obj_.detach(), probe_.detach(), rows_)
                    return errors.sum()

                @staticmethod
                def backward(ctx, grad_output):
                    obj_, probe_ = ctx.saved_tensors
                    need_probe = ctx.needs_input_grad[1]
                    _, g_obj, g_probe = ctx.model.loss_and_gradient(
                        obj_.detach(), probe_.detach(), ctx.rows, probe_gradient=need_probe)
                    g_obj = g_obj * grad_output if ctx.needs_input_grad[0] else None
                    if g_probe is not None:
                        g_probe = g_probe * grad_output
                    return g_obj, g_probe, None, None

            cls._cls = ForwardLoss
        return cls._cls.apply(obj, probe, model, rows)


def forward_model_loss(model: PtychoForwardModel, obj, probe, rows: Optional[object] = None):
    """Functional form of :meth:`PtychoForwardModel.loss`."""
    return model.loss(obj, probe, rows)
