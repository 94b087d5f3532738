"""NumPy restatement of the ptychographic-tomography loop of py4DSTEM 0.14.18.

TEST INFRASTRUCTURE ONLY: the CPU oracle the GPU tomography path is checked
against. Nothing in the product package imports it.

* ``spline_prefilter`` / ``rotate_volume``: _rotate_zxy_volume
  (ptychographic_methods.py:849-868), i.e. scipy.ndimage.affine_transform with
  order 3, mode "constant", prefilter on, restated: cubic B-spline coefficients
  by the recursive filter of Unser, Aldroubi & Eden (IEEE Trans. Signal Process.
  41, 1993) with the exact mirror-symmetric initial values, then the 4 x 4 x 4
  cubic B-spline sum at input coordinate offset + M o (0 outside [0, n - 1]).
* ``project_sliced`` / ``expand_sliced``: ptychographic_methods.py:783-847.
* ``TomographyOracle.reconstruct``: ptychographic_tomography.py:974-1240 for
  gradient descent, using the multislice primitives of ``oracle.ptycho_np``.
  The amplitudes stay float64 as the reference stores them
  (ptychographic_tomography.py:377-379, ``np.empty`` of float64), so the NumPy
  type promotions of the Fourier projection follow the reference's.

Pinned against tests/golden/tomo_*.npz, which the unmodified reference wrote.
"""

from __future__ import annotations

import numpy as np

from oracle.ptycho_np import Oracle, State

_SWAP_ZXY_TO_XYZ = np.array([[0, 1, 0], [0, 0, 1], [1, 0, 0]])
_POLE = np.sqrt(3.0) - 2.0


def _prefilter_axis(c: np.ndarray, axis: int) -> np.ndarray:
    x = np.moveaxis(c, axis, 0)
    n = x.shape[0]
    if n < 2:
        return c
    z = _POLE
    x *= (1.0 - z) * (1.0 - 1.0 / z)
    zl = z ** (n - 1)
    s = x[0] + zl * x[n - 1]
    zi = z
    for i in range(1, n - 1):
        s = s + zi * (x[i] + zl * x[n - 1 - i])
        zi *= z
    x[0] = s / (1.0 - zl * zl)
    for i in range(1, n):
        x[i] = x[i] + z * x[i - 1]
    x[n - 1] = (z * x[n - 2] + x[n - 1]) * z / (z * z - 1.0)
    for i in range(n - 2, -1, -1):
        x[i] = z * (x[i + 1] - x[i])
    return c


def spline_prefilter(volume: np.ndarray) -> np.ndarray:
    """Float64 cubic B-spline coefficients of `volume` (mirror-symmetric edges)."""
    c = np.array(volume, dtype=np.float64, copy=True)
    for axis in range(c.ndim):
        _prefilter_axis(c, axis)
    return c


def _mirror(i: np.ndarray, n: int) -> np.ndarray:
    if n == 1:
        return np.zeros_like(i)
    period = 2 * n - 2
    i = np.abs(i) % period
    return np.where(i >= n, period - i, i)


def _cubic_weights(t):
    u = 1.0 - t
    return [u * u * u / 6.0, 2.0 / 3.0 - t * t + t * t * t / 2.0,
            2.0 / 3.0 - u * u + u * u * u / 2.0, t * t * t / 6.0]


def affine_cubic(volume: np.ndarray, matrix: np.ndarray, offset: np.ndarray) -> np.ndarray:
    """affine_transform(volume, matrix, offset, order=3), output in volume's type."""
    shape = volume.shape
    c = spline_prefilter(volume)
    o = np.indices(shape, dtype=np.float64).reshape(3, -1)
    coords = []
    inside = np.ones(o.shape[1], dtype=bool)
    for h in range(3):
        v = np.full(o.shape[1], offset[h], dtype=np.float64)
        for l in range(3):
            v = v + matrix[h, l] * o[l]
        coords.append(v)
        inside &= ~(v < 0) & ~(v > shape[h] - 1)
    idx, w = [], []
    for h in range(3):
        x = coords[h][inside]
        f = np.floor(x)
        start = f.astype(np.int64) - 1
        w.append(_cubic_weights(x - f))
        idx.append([_mirror(start + k, shape[h]) for k in range(4)])
    value = np.zeros(int(inside.sum()), dtype=np.float64)
    for a in range(4):
        for b in range(4):
            wab = w[0][a] * w[1][b]
            for k in range(4):
                value = value + (wab * w[2][k]) * c[idx[0][a], idx[1][b], idx[2][k]]
    out = np.zeros(o.shape[1], dtype=np.float64)
    out[inside] = value
    return out.reshape(shape).astype(volume.dtype)


def rotation_transform(shape, rot_matrix):
    """(matrix, offset) of _rotate_zxy_volume for a volume of `shape`."""
    tf = _SWAP_ZXY_TO_XYZ.T @ rot_matrix.T @ _SWAP_ZXY_TO_XYZ
    in_center = (np.asarray(shape) - 1) / 2
    out_center = tf @ in_center
    return tf, in_center - out_center


def rotate_volume(volume: np.ndarray, rot_matrix: np.ndarray) -> np.ndarray:
    tf, offset = rotation_transform(volume.shape, rot_matrix)
    return affine_cubic(volume, tf, offset)


def project_sliced(volume: np.ndarray, num_slices: int) -> np.ndarray:
    """Sum of consecutive groups of ceil(Z / T) voxels along z, zero-padded."""
    z = volume.shape[0]
    vps = int(np.ceil(z / num_slices))
    out = np.empty((num_slices,) + volume.shape[1:], dtype=volume.dtype)
    for t in range(num_slices):
        s = None
        for k in range(vps):
            zz = t * vps + k
            v = volume[zz] if zz < z else np.zeros_like(volume[0])
            s = v.copy() if s is None else s + v
        out[t] = s
    return out


def expand_sliced(sliced: np.ndarray, num_voxels: int) -> np.ndarray:
    """Each slice divided by the voxels it covers (float64), repeated onto them."""
    t = sliced.shape[0]
    vps = int(np.ceil(num_voxels / t))
    rem = vps - (vps * t - num_voxels)
    counts = np.full(t, vps, dtype=np.int64)
    counts[-1] = rem if rem > 0 else vps
    norm = sliced / counts[:, None, None]
    return np.repeat(norm, vps, axis=0)[:num_voxels]


class TomographyOracle:
    """Reference tomography loop over preprocessed per-tilt state."""

    def __init__(self, *, volume, probes, amplitudes, positions_px, cum_counts, mean_intensity,
                 tilt_matrices, num_slices, propagators, fft_round_trip=False):
        """fft_round_trip: every FFT in complex128, rounded to complex64 (the
        same model under a more accurate float32 FFT; see Oracle)."""
        self.fft_round_trip = bool(fft_round_trip)
        self.volume = np.asarray(volume, dtype=np.float32).copy()
        self.probes = [np.asarray(p, dtype=np.complex64).copy() for p in probes]
        self.amplitudes = np.asarray(amplitudes, dtype=np.float64)
        self.positions_px = np.asarray(positions_px, dtype=np.float32).copy()
        self.cum = np.asarray(cum_counts)
        self.mean_intensity = list(mean_intensity)
        self.tilt_matrices = [np.asarray(m, dtype=np.float64) for m in tilt_matrices]
        self.num_slices = int(num_slices)
        self.propagators = np.asarray(propagators, dtype=np.complex64)
        self.error_iterations = []

    def _tilt_oracle(self, sliced, probe, index):
        start, end = self.cum[index], self.cum[index + 1]
        st = State(amplitudes=self.amplitudes[start:end].astype(np.float32),
                   positions_px=self.positions_px[start:end], probe=probe, object=sliced,
                   mean_intensity=float(self.mean_intensity[index]),
                   fov_mask_inverse=np.zeros(sliced.shape[-2:], dtype=bool),
                   object_type="potential", num_slices=self.num_slices,
                   propagators=self.propagators)
        o = Oracle(st, fft_round_trip=self.fft_round_trip)
        o.object = sliced  # work on the caller's arrays, as the reference does
        o.probe = probe
        return o

    def reconstruct(self, num_iter=8, max_batch_size=None, seed_random=None, step_size=0.5,
                    normalization_min=1.0, fix_probe=False, object_positivity=True,
                    shrinkage_rad=0.0, collective_measurement_updates=True,
                    detector_fourier_mask=None, gaussian_filter_sigma=None,
                    gaussian_filter=True, sampling=None):
        """gaussian_filter_sigma (A, with the real-space `sampling`): the volume's
        3D Gaussian blur (ptychographic_constraints.py:119-151 inside the 3D
        object constraints, :836-887), before shrinkage and positivity."""
        n_meas = len(self.tilt_matrices)
        total = int(self.cum[-1])
        if max_batch_size is not None:
            np.random.seed(seed_random)
        else:
            max_batch_size = total

        def constraints(vol):
            if gaussian_filter and gaussian_filter_sigma is not None:
                from scipy.ndimage import gaussian_filter as blur

                vol = blur(vol, gaussian_filter_sigma / sampling[0])
            if shrinkage_rad > 0.0:
                vol -= shrinkage_rad
            if object_positivity:
                vol = vol.clip(0.0)
            return vol

        for _ in range(num_iter):
            error = 0.0
            collective = np.zeros_like(self.volume) if collective_measurement_updates else None
            indices = np.arange(n_meas)
            np.random.shuffle(indices)
            old = np.eye(3)
            for index in indices:
                rot = self.tilt_matrices[index]
                self.volume = rotate_volume(self.volume, rot @ old.T)
                sliced = project_sliced(self.volume, self.num_slices)
                probe = self.probes[index]
                sliced_old = sliced.copy()
                start, end = int(self.cum[index]), int(self.cum[index + 1])
                n = end - start
                shuffled = np.arange(start, end)
                np.random.shuffle(shuffled)
                o = self._tilt_oracle(sliced, probe, index)
                measurement_error = 0.0
                for s, e in Oracle.batches(n, max_batch_size):
                    bi = shuffled[s:e]
                    pos = self.positions_px[bi]
                    frac = pos - np.round(pos)
                    rows, cols = o.patch_indices(pos)
                    amps = self.amplitudes[bi]
                    shifted = o.fft_shift(o.probe, frac)
                    shifted, patches, ov = o.overlap(rows, cols, shifted)
                    ew, be = o.gd_projection(amps, ov, detector_fourier_mask)
                    o.adjoint(patches, shifted, pos, ew, step_size, normalization_min, fix_probe,
                              False)
                    measurement_error += be
                sliced = o.object
                self.probes[index] = o.probe
                sliced -= sliced_old
                update = expand_sliced(sliced, self.volume.shape[0])
                if collective_measurement_updates:
                    collective += rotate_volume(update, rot.T)
                else:
                    self.volume += update
                old = rot
                measurement_error /= self.mean_intensity[index] * n
                error += measurement_error
                if not collective_measurement_updates:
                    self.volume = constraints(self.volume)
            self.volume = rotate_volume(self.volume, old.T)
            error /= n_meas
            if collective_measurement_updates:
                self.volume += collective / n_meas
                self.volume = constraints(self.volume)
            self.error_iterations.append(float(error))
        return self
