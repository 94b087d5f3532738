"""NumPy restatement of the py4DSTEM 0.14.18 ptychographic reconstruction loop.

TEST INFRASTRUCTURE ONLY (the parity oracle). The product package never imports
this module; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
do, and only to check or to time the CPU reference algorithm.

Input is the preprocessed state (corner-centred amplitudes, pixel positions,
initial object and probe, mean intensity, FOV mask); output is the object,
probe and error history after `num_iter` iterations. With dtype="float32" every
array operation follows the reference's own NumPy expressions in complex64 /
float32, so on the same inputs it reproduces the reference's CPU path; with
dtype="float64" the same model runs in complex128 / float64 (the FP64 evaluation
each GPU result is compared against).

Parity of this module is pinned by tests/golden/*.npz, which hold outputs of the
unmodified reference (tests/golden/make_golden.py) and are checked in
tests/test_oracle_golden.py.

Reference citations are py4DSTEM/process/phase/<file>:<line>.
"""

from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np


@dataclasses.dataclass
class State:
    """Preprocessed inputs of a reconstruction (what preprocess() leaves behind)."""

    amplitudes: np.ndarray          # (J, Sx, Sy) float32, corner-centred
    positions_px: np.ndarray        # (J, 2) float32
    probe: np.ndarray               # (Sx,Sy) or (M,Sx,Sy) complex64
    object: np.ndarray              # (Px,Py) / (T,Px,Py) complex64 or float32
    mean_intensity: float
    fov_mask_inverse: np.ndarray    # (Px,Py) bool
    object_type: str = "complex"
    num_slices: int = 1             # >1: multislice
    num_probes: int = 1             # >1 or mixed=True: mixed state
    mixed: bool = False
    propagators: Optional[np.ndarray] = None  # (T-1,Sx,Sy) complex64
    sampling: tuple = (1.0, 1.0)    # real-space pixel size (A), for position limits
    roi_shape: Optional[tuple] = None  # region_of_interest_shape; None: the detector's
    resample_exit_waves: bool = False  # set whenever region_of_interest_shape was given

    def copy(self):
        return dataclasses.replace(
            self, positions_px=self.positions_px.copy(), probe=self.probe.copy(),
            object=self.object.copy())


class Oracle:
    """Reference reconstruction loop over a :class:`State`."""

    def __init__(self, state: State, dtype: str = "float32", fft_round_trip: bool = False):
        """fft_round_trip=True evaluates every FFT in complex128 and rounds the
        result to the working precision: the same model with a different (more
        accurate) float32 FFT, used to measure how far the reference moves under
        FFT rounding alone."""
        if dtype not in ("float32", "float64"):
            raise ValueError("dtype must be 'float32' or 'float64'")
        self.fft_round_trip = fft_round_trip
        self.f = np.float32 if dtype == "float32" else np.float64
        self.c = np.complex64 if dtype == "float32" else np.complex128
        s = state
        self.amplitudes = np.asarray(s.amplitudes, dtype=self.f)
        self.positions_px = np.asarray(s.positions_px, dtype=np.float32).copy()
        self.positions_initial = self.positions_px.copy()
        self.sampling = tuple(s.sampling)
        self.object_type = s.object_type
        otype = self.f if s.object_type == "potential" else self.c
        self.object = np.asarray(s.object, dtype=otype).copy()
        self.probe = np.asarray(s.probe, dtype=self.c).copy()
        self.mean_intensity = s.mean_intensity
        self.fov_mask_inverse = np.asarray(s.fov_mask_inverse, dtype=bool)
        self.num_slices = s.num_slices
        self.mixed = s.mixed or s.num_probes > 1
        self.num_probes = s.num_probes
        self.propagators = (None if s.propagators is None
                            else np.asarray(s.propagators, dtype=self.c))
        self.amp_shape = np.array(self.amplitudes.shape[-2:])
        self.roi = np.array(s.roi_shape) if s.roi_shape is not None else self.amp_shape
        self.resample = bool(s.resample_exit_waves)
        self.object_shape = self.object.shape[-2:]
        self.J = self.amplitudes.shape[0]
        self.exit_waves = None
        self.error_iterations = []
        # Fourier amplitude of the initial probe (preprocess, store_initial_arrays)
        self.probe_initial_aperture = np.abs(np.fft.fft2(self.probe))

    def fft2(self, a):
        if self.fft_round_trip:
            return np.fft.fft2(a.astype(np.complex128)).astype(self.c)
        return np.fft.fft2(a)

    def ifft2(self, a):
        if self.fft_round_trip:
            return np.fft.ifft2(a.astype(np.complex128)).astype(self.c)
        return np.fft.ifft2(a)

    # ------------------------------------------------------------ A4, A5, A6, A15
    @staticmethod
    def batches(num_items, max_batch):
        """utils.py:539-589."""
        nb = (num_items + (-num_items % max_batch)) // max_batch
        if num_items % nb == 0:
            sizes = [num_items // nb] * nb
        else:
            zp = nb - (num_items % nb)
            pp = num_items // nb
            sizes = []
            for i in range(nb):
                sizes = ([pp + 1] if i >= zp else [pp]) + sizes
        start = 0
        for n in sizes:
            yield start, start + n
            start += n

    def patch_indices(self, positions_px):
        """phase_base_class.py:1970-2003."""
        x0 = np.round(positions_px[:, 0]).astype("int")
        y0 = np.round(positions_px[:, 1]).astype("int")
        xi = np.fft.fftfreq(self.roi[0], d=1 / self.roi[0]).astype("int")
        yi = np.fft.fftfreq(self.roi[1], d=1 / self.roi[1]).astype("int")
        rows = (x0[:, None, None] + xi[None, :, None]) % self.object_shape[0]
        cols = (y0[:, None, None] + yi[None, None, :]) % self.object_shape[1]
        return rows, cols

    def fft_shift(self, array, positions):
        """utils.py:468-533."""
        f = self.f
        kx = np.fft.fftfreq(array.shape[-2], 1.0).astype(f)
        ky = np.fft.fftfreq(array.shape[-1], 1.0).astype(f)
        pos = np.asarray(positions, dtype=f)
        single = pos.ndim == 1
        if single:
            pos = pos[None]
        x = pos[:, 0].ravel()[:, None, None]
        y = pos[:, 1].ravel()[:, None, None]
        op = np.exp(-2.0j * np.pi * kx[None, :, None] * x) * np.exp(
            -2.0j * np.pi * ky[None, None, :] * y)
        if single:
            op = op[0]
        fa = self.fft2(array)
        if op.ndim == 3 and fa.ndim == 3:
            shifted = fa[None] * op[:, None]
        else:
            shifted = fa * op
        return self.ifft2(shifted)

    def scatter(self, patches, positions_px):
        """phase_base_class.py:1905-1968 (float64 bincount, then float32/64)."""
        if np.iscomplexobj(patches):
            return self._scatter_real(patches.real, positions_px) + 1.0j * self._scatter_real(
                patches.imag, positions_px)
        return self._scatter_real(patches, positions_px)

    def _scatter_real(self, patches, positions_px):
        x0 = np.round(positions_px[:, 0]).astype("int")
        y0 = np.round(positions_px[:, 1]).astype("int")
        xi = np.fft.fftfreq(self.roi[0], d=1 / self.roi[0]).astype("int")
        yi = np.fft.fftfreq(self.roi[1], d=1 / self.roi[1]).astype("int")
        shape = self.object_shape
        idx = ((y0[:, None, None] + yi[None, None, :]) % shape[1]) + (
            (x0[:, None, None] + xi[None, :, None]) % shape[0]) * shape[1]
        counts = np.bincount(idx.ravel(), weights=patches.ravel(), minlength=int(np.prod(shape)))
        return np.reshape(counts, shape).astype(self.f)

    # ------------------------------------------------------------- forward A7-A12
    def overlap(self, rows, cols, shifted):
        """ptychographic_methods.py:1489-1527 (2D), 2300-2351 (2.5D), 2696-2734 (mixed),
        3102-3160 (2.5D mixed)."""
        if self.num_slices > 1 and self.mixed:
            patches = self.object[:, rows, cols]
            if self.object_type == "potential":
                patches = np.exp(1j * patches)
            # (T, B, M, Sx, Sy); an unshifted (M, Sx, Sy) probe broadcasts over B
            shape = (self.num_slices, patches.shape[1], self.num_probes) + patches.shape[-2:]
            probes = np.empty(shape, dtype=patches.dtype)
            probes[0] = shifted
            for s in range(self.num_slices):
                ov = np.expand_dims(patches[s], axis=1) * probes[s]
                if s + 1 < self.num_slices:
                    probes[s + 1] = self.ifft2(self.fft2(ov) * self.propagators[s])
            return probes, patches, ov
        if self.num_slices > 1:
            patches = self.object[:, rows, cols]
            if self.object_type == "potential":
                patches = np.exp(1j * patches)
            probes = np.empty_like(patches)
            probes[0] = shifted
            for s in range(self.num_slices):
                ov = patches[s] * probes[s]
                if s + 1 < self.num_slices:
                    probes[s + 1] = self.ifft2(self.fft2(ov) * self.propagators[s])
            return probes, patches, ov
        patches = self.object[rows, cols]
        if self.object_type == "potential":
            patches = np.exp(1j * patches)
        if self.mixed:
            return shifted, patches, shifted * np.expand_dims(patches, axis=1)
        return shifted, patches, shifted * patches

    @staticmethod
    def bilinear_resample(array, output_size):
        """utils.py:2347-2428 (vectorized, conserve_array_sums=True): scipy.ndimage.zoom
        with order 1, mode "grid-wrap", grid_mode=True over the last two axes,
        divided by the ratio of pixel counts (a float64 scalar: complex64 input
        comes back complex128, as in the reference)."""
        from scipy.ndimage import zoom

        input_size = np.array(array.shape[-2:])
        scale = tuple(np.array(output_size) / input_size)
        scale = (1,) * (array.ndim - 2) + scale
        out = zoom(array, scale, order=1, mode="grid-wrap", grid_mode=True)
        return out / np.array(scale).prod()

    def to_detector(self, fo):
        """ptychographic_methods.py:1601-1609: resample to match the data."""
        return self.bilinear_resample(fo, self.amp_shape) if self.resample else fo

    def to_roi(self, fo):
        """ptychographic_methods.py:1623-1631: back to region_of_interest_shape."""
        return self.bilinear_resample(fo, self.roi) if self.resample else fo

    def farfield(self, fo):
        if self.mixed:
            return np.sqrt(np.sum(np.abs(fo) ** 2, axis=1))
        return np.abs(fo)

    def gd_projection(self, amplitudes, overlap, mask):
        """ptychographic_methods.py:1576-1635 and 2742-2804."""
        fo = self.to_detector(self.fft2(overlap))
        if mask is not None:
            fo *= mask
        ff = self.farfield(fo)
        error = np.sum(np.abs(amplitudes - ff) ** 2)
        if self.mixed:
            ff[ff == 0.0] = np.inf
            mod = (amplitudes / ff)[:, None] * fo - fo
        else:
            mod = amplitudes * np.exp(1j * np.angle(fo)) - fo
        if mask is not None:
            mod *= mask
        return self.ifft2(self.to_roi(mod)), error

    def ps_projection(self, amplitudes, overlap, exit_waves, a, b, c):
        """ptychographic_methods.py:1637-1734 and 2806-2904."""
        x = 1 - a - b
        y = 1 - c
        if exit_waves is None:
            exit_waves = overlap.copy()
        factor = c * overlap + y * exit_waves
        fp = self.to_detector(self.fft2(factor))
        ff = self.farfield(fp)
        error = np.sum(np.abs(amplitudes - ff) ** 2)
        if self.mixed:
            ff[ff == 0.0] = np.inf
            fp *= (amplitudes / ff)[:, None]
        else:
            fp = amplitudes * np.exp(1j * np.angle(fp))
        projected = self.ifft2(self.to_roi(fp))
        return x * exit_waves + a * overlap + b * projected, error

    # --------------------------------------------------------------- adjoint A13-A14
    def _normaliser(self, s, m):
        return 1 / np.sqrt(1e-16 + ((1 - m) * s) ** 2 + (m * np.max(s)) ** 2)

    def _obj_term(self, patch, probe, chi):
        if self.object_type == "potential":
            return np.real(-1j * np.conj(patch) * np.conj(probe) * chi)
        return np.conj(probe) * chi

    def adjoint(self, patches, shifted, positions_px, ew, step, m, fix_probe, projection):
        """ptychographic_methods.py:1818-2069 (2D), 2353-2565 (2.5D), 2906-3093 (mixed),
        3162-3340 (2.5D mixed)."""
        obj, probe = self.object, self.probe
        if self.num_slices > 1 and self.mixed:
            ew = ew.copy() if projection else ew
            for s in reversed(range(self.num_slices)):
                pr = shifted[s]
                op = patches[s]
                pn = np.zeros_like(obj[s])
                upd = np.zeros_like(obj[s])
                for i in range(self.num_probes):
                    pn += self.scatter(np.abs(pr[:, i]) ** 2, positions_px)
                    term = self.scatter(self._obj_term(op, pr[:, i], ew[:, i]), positions_px)
                    upd += term if projection else step * term
                pn = self._normaliser(pn, m)
                if projection:
                    obj[s] = upd * pn
                else:
                    obj[s] += upd * pn
                ew *= np.expand_dims(np.conj(op), axis=1)
                if s > 0:
                    ew = self.ifft2(self.fft2(ew) * np.conj(self.propagators[s - 1]))
                elif not fix_probe:
                    on = self._normaliser(np.sum(np.abs(op) ** 2, axis=0), m)
                    if projection:
                        probe = np.sum(ew, axis=0) * on[None]
                    else:
                        probe += step * np.sum(ew, axis=0) * on[None]
            self.object, self.probe = obj, probe
            return
        if self.num_slices > 1:
            ew = ew.copy() if projection else ew
            for s in reversed(range(self.num_slices)):
                pr = shifted[s]
                op = patches[s]
                nrm = self._normaliser(self.scatter(np.abs(pr) ** 2, positions_px), m)
                upd = self.scatter(self._obj_term(op, pr, ew), positions_px) * nrm
                if projection:
                    obj[s] = upd
                else:
                    obj[s] += step * upd
                ew *= np.conj(op)
                if s > 0:
                    ew = self.ifft2(self.fft2(ew) * np.conj(self.propagators[s - 1]))
                elif not fix_probe:
                    on = self._normaliser(np.sum(np.abs(op) ** 2, axis=0), m)
                    if projection:
                        probe = np.sum(ew, axis=0) * on
                    else:
                        probe += step * np.sum(ew, axis=0) * on
            self.object, self.probe = obj, probe
            return
        if self.mixed:
            pn = np.zeros_like(obj)
            upd = np.zeros_like(obj)
            for i in range(self.num_probes):
                pn += self.scatter(np.abs(shifted[:, i]) ** 2, positions_px)
                term = self.scatter(self._obj_term(patches, shifted[:, i], ew[:, i]), positions_px)
                upd += term if projection else step * term
            pn = self._normaliser(pn, m)
            if projection:
                obj = upd * pn
            else:
                obj += upd * pn
            if not fix_probe:
                on = self._normaliser(np.sum(np.abs(patches) ** 2, axis=0), m)
                g = np.sum(np.expand_dims(np.conj(patches), axis=1) * ew, axis=0) * on[None]
                if projection:
                    probe = g
                else:
                    probe += step * g  # in place, :2992 (a complex128 term is cast back)
            self.object, self.probe = obj, probe
            return
        pn = self._normaliser(self.scatter(np.abs(shifted) ** 2, positions_px), m)
        upd = self.scatter(self._obj_term(patches, shifted, ew), positions_px) * pn
        if projection:
            obj = upd
        else:
            obj += step * upd
        if not fix_probe:
            on = self._normaliser(np.sum(np.abs(patches) ** 2, axis=0), m)
            g = np.sum(np.conj(patches) * ew, axis=0) * on
            if projection:
                probe = g
            else:
                probe += step * g  # in place, :1900
        self.object, self.probe = obj, probe

    # ------------------------------------------------------- position correction A16
    def position_correction(self, rows, cols, shifted, ov, amps, pos, pos_init, step,
                            max_update, max_total):
        """ptychographic_methods.py:2071-2225 (far fields resampled to the detector
        as at :2119-2173 when region_of_interest_shape was given): a
        per-position 2x2 least-squares shift from the intensity change of one-pixel
        object shifts, computed with the object after this batch's update, the
        overlap of the forward pass and `shifted` (the forward pass's shifted probes,
        or for multislice the updated probe)."""
        fo = self.to_detector(self.fft2(ov))
        fo_conj = np.conj(fo)
        estimated = self.farfield(fo) ** 2
        measured = amps ** 2
        flat = (measured.shape[0], -1)
        difference = (measured - estimated).reshape(flat)
        _, _, ov_dx = self.overlap((rows + 1) % self.object_shape[0], cols, shifted)
        _, _, ov_dy = self.overlap(rows, (cols + 1) % self.object_shape[1], shifted)
        fdx = fo - self.to_detector(self.fft2(ov_dx))
        fdy = fo - self.to_detector(self.fft2(ov_dy))
        pdx = 2 * np.real(fdx * fo_conj)
        pdy = 2 * np.real(fdy * fo_conj)
        if pdx.ndim == 4:
            pdx = pdx.sum(1)
            pdy = pdy.sum(1)
        pdx = pdx.reshape(flat)
        pdy = pdy.reshape(flat)
        cm = np.dstack((pdx, pdy))
        cm_t = cm.conj().swapaxes(-1, -2)
        update = np.linalg.inv(cm_t @ cm) @ cm_t @ difference[..., None]
        update = update[..., 0] * step
        scale = np.sqrt(self.sampling[0] ** 2 + self.sampling[1] ** 2)
        if max_update is not None:
            max_update = max_update / scale
            norms = np.linalg.norm(update, axis=1)
            out = norms > max_update
            update[out] /= norms[out, None] / max_update
        if max_total is not None:
            max_total = max_total / scale
            deltas = (pos - pos_init) - update
            out = np.linalg.norm(deltas, axis=1) > max_total
            update[out] = 0
        pos -= update
        return pos

    def positions_com_constraint(self):
        """ptychographic_constraints.py:1292-1311."""
        self.positions_px -= self.positions_px.mean(0) - self.positions_initial.mean(0)

    # affine map x -> (x - o) @ M + t + o with M = scale @ shear @ rotation
    # (utils.py:580-741); (scale0, scale1, shear1, angle, t0, t1)
    @staticmethod
    def _affine_apply(p, x, origin):
        origin = np.asarray(origin, dtype=np.float32)
        c, s = np.cos(p[3]), np.sin(p[3])
        m = (np.array([[p[0], 0.0], [0.0, p[1]]], dtype="float32")
             @ np.array([[1.0, 0.0], [p[2], 1.0]], dtype="float32")
             @ np.array([[+c, -s], [+s, +c]], dtype="float32"))
        return ((x - origin) @ np.asarray(m, dtype=np.float32)) + (np.array((p[4], p[5]))
                                                                   + origin)

    @classmethod
    def _affine_fit(cls, x0, x1, origin):
        """utils.py:743-770 (translation allowed) with AffineTransform.fromarray
        (utils.py:640-671)."""
        identity = (1.0, 1.0, 0.0, 0.0, 0.0, 0.0)
        origin = np.asarray(origin, dtype=np.float32)
        try:
            a = np.pad(x0 - origin, ((0, 0), (0, 1)), constant_values=1)
            aT = a.conj().swapaxes(-1, -2)
            T = np.linalg.inv(aT @ a) @ aT @ (x1 - origin)
            R = T[:2, :2].copy()
            s0 = np.linalg.norm(R[0])
            p = identity
            if s0 > 0:
                R[0] /= s0
                sh = R[0] @ R[1]
                R[1] -= sh * R[0]
                s1 = np.linalg.norm(R[1])
                if s1 > 0:
                    R[1] /= s1
                    sh /= s1
                    p = (float(s0), float(s1), float(sh), float(np.arccos(R[0, 0])),
                         T[2][0], T[2][1])
        except np.linalg.LinAlgError:
            p = identity
        return p, np.linalg.norm(cls._affine_apply(p, x0, origin) - x1)

    def positions_affine_constraint(self):
        """ptychographic_constraints.py:1313-1350 with the RANSAC of utils.py:773-827
        (20 subsets of J // 10 indices from the global generator, inliers within
        16 px, consensus 0.75)."""
        x0, x1 = self.positions_initial, self.positions_px
        com = x0.mean(0)
        best, params = np.inf, (1.0, 1.0, 0.0, 0.0, 0.0, 0.0)
        for subset in np.random.choice(a=len(x0), size=(20, x0.shape[0] // 10), replace=True):
            subset = np.unique(subset)
            p, _ = self._affine_fit(x0[subset], x1[subset], com)
            inl = np.linalg.norm(self._affine_apply(p, x0, com) - x1, axis=-1) <= 16
            if np.sum(inl) / len(inl) >= 0.75:
                p, fit = self._affine_fit(x0[inl], x1[inl], com)
                if fit < best:
                    best, params = fit, p
        self.positions_px = self._affine_apply(params, x0, com)

    # ------------------------------------------------------- self-consistency A19
    def self_consistency_errors(self, max_batch_size=None):
        """ptychographic_methods.py:2227-2291: per-position sum (A - |F|)^2 of a
        forward-only pass in natural order, divided by the mean intensity."""
        if max_batch_size is None:
            max_batch_size = self.J
        errors = np.array([])
        for start, end in self.batches(self.J, max_batch_size):
            pos = self.positions_px[start:end]
            frac = pos - np.round(pos)
            rows, cols = self.patch_indices(pos)
            shifted = self.fft_shift(self.probe, frac)
            _, _, ov = self.overlap(rows, cols, shifted)
            ff = self.farfield(self.to_detector(self.fft2(ov)))
            errors = np.hstack((errors, np.sum(np.abs(self.amplitudes[start:end] - ff) ** 2,
                                               axis=(-2, -1))))
        errors /= self.mean_intensity
        return errors

    # ------------------------------------------------------------ constraints A17
    def object_constraints(self, shrinkage_rad, mask, pure_phase, positivity):
        """ptychographic_constraints.py:29-117, 411-464, 649-726 (default-on subset)."""
        o = self.object
        if shrinkage_rad > 0.0 or mask is not None:
            if self.object_type == "complex":
                phase = np.angle(o)
                amp = np.abs(o)
                if mask is not None:
                    shrinkage_rad += phase[..., mask].mean()
                phase -= shrinkage_rad
                o = amp * np.exp(1.0j * phase)
            else:
                if mask is not None:
                    shrinkage_rad += o[..., mask].mean()
                o -= shrinkage_rad
        if self.object_type == "complex":
            phase = np.angle(o)
            amp = 1.0 if pure_phase else np.minimum(np.abs(o), 1.0)
            o = amp * np.exp(1.0j * phase)
        elif positivity:
            o = o.clip(0.0)
        self.object = o

    def center_of_mass(self, ar):
        """process/utils/utils.py:166-187 (corner-centred)."""
        nx, ny = ar.shape
        ry, rx = np.meshgrid(np.fft.fftfreq(ny, 1 / ny), np.fft.fftfreq(nx, 1 / nx))
        tot = np.sum(ar)
        return np.sum(rx * ar) / tot, np.sum(ry * ar) / tot

    def probe_com_constraint(self):
        """ptychographic_constraints.py:894-918, 1156-1179."""
        inten = np.abs(self.probe[0] if self.mixed else self.probe) ** 2
        x0, y0 = self.center_of_mass(inten)
        self.probe = self.fft_shift(self.probe, -np.array([x0, y0]))

    def object_gaussian(self, sigma_px, pure_phase):
        """ptychographic_constraints.py:119-151."""
        from scipy.ndimage import gaussian_filter

        if not pure_phase or self.object_type == "potential":
            self.object = gaussian_filter(self.object, sigma_px)
        else:
            phase = gaussian_filter(np.angle(self.object), sigma_px)
            self.object = np.exp(1.0j * phase)

    def object_identical_slices(self):
        """ptychographic_constraints.py:630-647."""
        self.object[:] = self.object.mean(0, keepdims=True)

    @staticmethod
    def _probe_aperture(p, aperture):
        """ptychographic_constraints.py:1004-1040."""
        s0 = np.sum(np.abs(p) ** 2)
        phase = np.angle(np.fft.fft2(p))
        u = np.fft.ifft2(np.exp(1j * phase) * aperture)
        return u * np.sqrt(s0 / np.sum(np.abs(u) ** 2))

    @staticmethod
    def _probe_amplitude(p, relative_radius, relative_width):
        """ptychographic_constraints.py:920-957."""
        from scipy.special import erf

        s0 = np.sum(np.abs(p) ** 2)
        X = np.fft.fftfreq(p.shape[0])[:, None]
        Y = np.fft.fftfreq(p.shape[1])[None]
        r = np.hypot(X, Y) - relative_radius
        sigma = np.sqrt(np.pi) / relative_width
        u = p * (0.5 * (1 - erf(sigma * r / (1 - r ** 2))))
        return u * np.sqrt(s0 / np.sum(np.abs(u) ** 2))

    def probe_optional_constraints(self, aperture, amplitude, radius, width):
        """ptychographic_constraints.py:1091-1148 (single probe), 1218-1285 (mixed)."""
        if aperture:
            if self.mixed:
                self.probe[0] = self._probe_aperture(self.probe[0],
                                                     self.probe_initial_aperture[0])
            else:
                self.probe = self._probe_aperture(self.probe, self.probe_initial_aperture)
        if amplitude:
            if self.mixed:
                for i in range(self.num_probes):
                    self.probe[i] = self._probe_amplitude(self.probe[i], radius, width)
            else:
                self.probe = self._probe_amplitude(self.probe, radius, width)

    def probe_orthogonalization(self):
        """ptychographic_constraints.py:1181-1216."""
        n = self.num_probes
        p = self.probe
        gram = np.empty((n, n), dtype=p.dtype)
        for i in range(n):
            for j in range(i, n):
                gram[i, j] = np.sum(p[i].conj() * p[j])
        _, evecs = np.linalg.eigh(gram, UPLO="U")
        p = np.tensordot(evecs.T, p, axes=1)
        inten = np.sum(np.abs(p) ** 2, axis=(-2, -1))
        self.probe = p[np.argsort(inten, axis=None)[::-1]]

    # ---------------------------------------------------------------- loop A1-A3
    def reconstruct(self, num_iter=8, method="GD", a=None, b=None, c=None, max_batch_size=None,
                    seed_random=None, step_size=0.5, normalization_min=1.0, fix_probe=False,
                    fix_probe_com=True, orthogonalize_probe=True, shrinkage_rad=0.0,
                    fix_potential_baseline=True, pure_phase_object=False,
                    object_positivity=True, detector_fourier_mask=None, fix_positions=True,
                    fix_positions_com=True, positions_step_size=0.5,
                    max_position_update_distance=None, max_position_total_distance=None,
                    fix_probe_aperture=False, constrain_probe_amplitude=False,
                    constrain_probe_amplitude_relative_radius=0.5,
                    constrain_probe_amplitude_relative_width=0.05, identical_slices=False,
                    gaussian_filter_sigma=None, gaussian_filter=True,
                    global_affine_transformation=False):
        """singleslice_ptychography.py:606-996 (and the multislice / mixed-state twins)."""
        projection = method != "GD"
        J = self.J
        order = np.arange(J)
        if max_batch_size is not None:
            np.random.seed(seed_random)
        else:
            max_batch_size = J
        mask = (self.fov_mask_inverse
                if fix_potential_baseline and self.fov_mask_inverse.sum() > 0 else None)
        error = None
        for _ in range(num_iter):
            error = 0.0
            if not projection:
                np.random.shuffle(order)
            for start, end in self.batches(J, max_batch_size):
                idx = order[start:end]
                pos = self.positions_px[idx]
                frac = pos - np.round(pos)
                rows, cols = self.patch_indices(pos)
                amps = self.amplitudes[idx]
                shifted = self.fft_shift(self.probe, frac)
                shifted, patches, ov = self.overlap(rows, cols, shifted)
                if projection:
                    self.exit_waves, be = self.ps_projection(amps, ov, self.exit_waves, a, b, c)
                    ew = self.exit_waves
                else:
                    ew, be = self.gd_projection(amps, ov, detector_fourier_mask)
                self.adjoint(patches, shifted, pos, ew, step_size, normalization_min, fix_probe,
                             projection)
                if not fix_positions:
                    # multislice passes the updated, unshifted probe
                    # (multislice_ptychography.py:1026-1038)
                    self.positions_px[idx] = self.position_correction(
                        rows, cols, self.probe if self.num_slices > 1 else shifted, ov, amps,
                        pos, self.positions_initial[idx],
                        positions_step_size, max_position_update_distance,
                        max_position_total_distance)
                error += be
            error /= self.mean_intensity * J
            if gaussian_filter and gaussian_filter_sigma is not None:
                self.object_gaussian(gaussian_filter_sigma / self.sampling[0],
                                     pure_phase_object and self.object_type == "complex")
            if identical_slices and self.num_slices > 1:
                self.object_identical_slices()
            self.object_constraints(shrinkage_rad, mask,
                                    pure_phase_object and self.object_type == "complex",
                                    object_positivity)
            if fix_probe_com and not fix_probe:
                self.probe_com_constraint()
            self.probe_optional_constraints(
                fix_probe_aperture and not fix_probe, constrain_probe_amplitude and not fix_probe,
                constrain_probe_amplitude_relative_radius, constrain_probe_amplitude_relative_width)
            if self.mixed and orthogonalize_probe:
                self.probe_orthogonalization()
            # phase_base_class.py:2179-2195 passes fix_positions_com and not fix_positions
            if not fix_positions and not (fix_positions_com and not fix_positions):
                self.positions_com_constraint()
            if not fix_positions and global_affine_transformation:
                self.positions_affine_constraint()
            self.error_iterations.append(float(error))
        return self

    # ---------------------------------------------------- single-batch primitives
    def forward_batch(self, idx):
        """Forward model of one batch (no update): returns (shifted probes, patches,
        exit waves, chi, error) for kernel-level parity tests."""
        pos = self.positions_px[idx]
        frac = pos - np.round(pos)
        rows, cols = self.patch_indices(pos)
        shifted = self.fft_shift(self.probe, frac)
        shifted, patches, ov = self.overlap(rows, cols, shifted)
        chi, err = self.gd_projection(self.amplitudes[idx], ov, None)
        return shifted, patches, ov, chi, err


def method_abc(method, parameter=1.0, a=None, b=None, c=None):
    """phase_base_class.py:2005-2108: projection parameters of a named method."""
    if method in ("GD", "gradient-descent"):
        return "GD", None, None, None
    if method in ("DM_AP", "difference-map_alternating-projections"):
        return "PS", -parameter, 1, 1 + parameter
    if method in ("RAAR", "relaxed-averaged-alternating-reflections"):
        return "PS", 1 - 2 * parameter, parameter, 2
    if method in ("RRR", "relax-reflect-reflect"):
        return "PS", -parameter, parameter, 2
    if method in ("SUPERFLIP", "charge-flipping"):
        return "PS", 0, 1, 2
    if method == "generalized-projections":
        return "PS", a, b, c
    raise ValueError(method)
