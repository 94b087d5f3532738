"""Host-side preprocessing shared by the three reconstruction classes.

This is the one-time setup before the GPU hot loop: calibrations, diffraction
centre of mass and its plane fit, the real/reciprocal rotation search, corner
centring and square-root of the patterns, scan positions in object pixels, and
the initial object, probe and field-of-view mask. It runs on the host with NumPy
in float32/complex64, step for step like the reference so that the arrays
handed to the GPU are the reference's arrays:

=========================================  =============================================
step                                       reference (py4DSTEM 0.14.18)
=========================================  =============================================
datacube padding / binning                 phase_base_class.py:223-422
intensities and calibrations               phase_base_class.py:424-611
vectorised centre of mass + plane fit      phase_base_class.py:613-767, calibration/origin.py:76-190
rotation / transpose (curl or divergence)  phase_base_class.py:769-1345
bilinear corner-centring, sqrt, mean I     phase_base_class.py:1347-1460, preprocess/utils.py:59-120
scan positions in pixels                   phase_base_class.py:1811-1903
object / probe initialisation              ptychographic_methods.py:40-79, 403-443, 1011-1102, 1416-1462
probe overlap and FOV mask                 singleslice_ptychography.py:504-540
=========================================  =============================================

Nothing here is on the per-position path; the reconstruction loop itself runs in
libptycho_gb300 (see engine.py).
"""

from __future__ import annotations

import warnings
from inspect import signature

import numpy as np
from scipy.ndimage import gaussian_filter
from scipy.optimize import curve_fit

from .optics import ComplexProbe, electron_wavelength_angstrom


def bilinear_resample(array, output_size, conserve_array_sums=False):
    """Resize the last two axes by linear interpolation on a periodic grid
    (utils.py:2347-2428 with vectorized=True): scipy.ndimage.zoom with order 1,
    mode "grid-wrap" and grid_mode=True, the leading axes kept; divided by the
    ratio of pixel counts when conserve_array_sums. Host-side, once per
    reconstruction (the vacuum probe); the reconstruction kernels resample the
    far fields themselves."""
    from scipy.ndimage import zoom

    array = np.asarray(array)
    input_size = np.array(array.shape[-2:])
    output_size = np.array(output_size)
    scale = tuple(output_size / input_size)
    scale = (1,) * (array.ndim - 2) + scale
    out = zoom(array, scale, order=1, mode="grid-wrap", grid_mode=True)
    if conserve_array_sums:
        out = out / np.array(scale).prod()
    return out

# ----------------------------------------------------------------- small helpers


def generate_batches(num_items: int, max_batch: int):
    """Yield (start, end) of near-equal batches (utils.py:539-589): the
    `num_items % num_batches` batches that get one extra item come first."""
    num_batches = (num_items + (-num_items % max_batch)) // max_batch
    if num_items < num_batches:
        raise RuntimeError("num_batches may not be larger than num_items")
    if num_items % num_batches == 0:
        sizes = [num_items // num_batches] * num_batches
    else:
        small = num_batches - (num_items % num_batches)
        base = num_items // num_batches
        sizes = [base + 1] * (num_batches - small) + [base] * small
    start = 0
    for size in sizes:
        yield start, start + size
        start += size


def center_of_mass(ar, corner_centered=False):
    """Intensity centre of mass in pixels (process/utils/utils.py:166-187)."""
    ar = np.asarray(ar)
    nx, ny = ar.shape
    if corner_centered:
        ry, rx = np.meshgrid(np.fft.fftfreq(ny, 1 / ny), np.fft.fftfreq(nx, 1 / nx))
    else:
        ry, rx = np.meshgrid(np.arange(ny), np.arange(nx))
    tot = np.sum(ar)
    return np.sum(rx * ar) / tot, np.sum(ry * ar) / tot


def shift_bilinear(ar, xshift, yshift):
    """Periodic bilinear shift of a 2D array (preprocess/utils.py:59-120,
    bilinear branch)."""
    xf = int(np.floor(xshift))
    yf = int(np.floor(yshift))
    wx = xshift - xf
    wy = yshift - yf
    return (
        np.roll(ar, (xf, yf), axis=(0, 1)) * ((1 - wx) * (1 - wy))
        + np.roll(ar, (xf + 1, yf), axis=(0, 1)) * (wx * (1 - wy))
        + np.roll(ar, (xf, yf + 1), axis=(0, 1)) * ((1 - wx) * wy)
        + np.roll(ar, (xf + 1, yf + 1), axis=(0, 1)) * (wx * wy)
    )


def _corner_slices(n_in, n_out):
    """(source, destination) index slices of the two corners of a spectrum axis
    that a Fourier resize keeps: the first ceil(m/2) and the last floor(m/2)
    frequencies, m = min(n_in, n_out); the whole axis when the sizes agree."""
    if n_in == n_out:
        return (slice(None), slice(None)), (slice(None), slice(None))
    m = min(n_in, n_out)
    lo, hi = (m + 1) // 2, m // 2
    return (slice(0, lo), slice(0, lo)), (slice(n_in - hi, n_in), slice(n_out - hi, n_out))


def fourier_resample(array, output_size, force_nonnegative=False, conserve_array_sums=True,
                     chunk=256):
    """Fourier interpolation of the last two axes of a 2D or 4D array to
    `output_size` (process/utils/utils.py:412-640): the kept corners of each
    pattern's complex64 spectrum are copied into a zero spectrum of the new
    size, inverse transformed, and the real part taken as float32; negative
    values clipped when force_nonnegative; multiplied by the size ratio unless
    conserve_array_sums."""
    array = np.asarray(array)
    n_in = array.shape[-2:]
    output_size = tuple(int(v) for v in output_size)
    (xa, xb), (xc, xd) = _corner_slices(n_in[0], output_size[0])
    (ya, yb), (yc, yd) = _corner_slices(n_in[1], output_size[1])
    corners = [((xa, ya), (xb, yb)), ((xc, ya), (xd, yb)), ((xa, yc), (xb, yd)),
               ((xc, yc), (xd, yd))]

    def resize(block):
        spec = np.fft.fft2(block)
        out = np.zeros(block.shape[:-2] + output_size, dtype=np.complex64)
        for (sx_, sy_), (dx_, dy_) in corners:
            out[..., dx_, dy_] = spec[..., sx_, sy_]
        return np.real(np.fft.ifft2(out)).astype(np.float32)

    if array.ndim == 2:
        result = resize(array)
    elif array.ndim == 4:
        result = np.zeros(array.shape[:2] + output_size, dtype=np.float32)
        flat_in = array.reshape((-1,) + n_in)
        flat_out = result.reshape((-1,) + output_size)
        for start in range(0, flat_in.shape[0], chunk):
            flat_out[start:start + chunk] = resize(flat_in[start:start + chunk])
    else:
        raise ValueError(f"fourier_resample takes 2D or 4D arrays, not {array.ndim}D")
    if force_nonnegative:
        result = np.maximum(result, 0)
    if not conserve_array_sums:
        result = result * (np.prod(output_size) / np.prod(n_in))
    return result


def _plane(xy, mx, my, b):
    return mx * xy[0] + my * xy[1] + b


def _parabola(xy, c0, cx1, cx2, cy1, cy2, cxy):
    return c0 + cx1 * xy[0] + cy1 * xy[1] + cx2 * xy[0] ** 2 + cy2 * xy[1] ** 2 + cxy * xy[0] * xy[1]


def _bezier_two(xy, c00, c01, c02, c10, c11, c12, c20, c21, c22):
    u, v = xy[0], xy[1]
    return (
        c00 * ((1 - u) ** 2) * ((1 - v) ** 2)
        + c10 * 2 * (1 - u) * u * ((1 - v) ** 2)
        + c20 * (u**2) * ((1 - v) ** 2)
        + c01 * 2 * ((1 - u) ** 2) * (1 - v) * v
        + c11 * 4 * (1 - u) * u * (1 - v) * v
        + c21 * 2 * (u**2) * (1 - v) * v
        + c02 * ((1 - u) ** 2) * (v**2)
        + c12 * 2 * (1 - u) * u * (v**2)
        + c22 * (u**2) * (v**2)
    )


_FIT_FUNCTIONS = {"plane": _plane, "parabola": _parabola, "bezier_two": _bezier_two}


def _fit_surface(function, data, mask):
    """Least-squares surface fit over unit-square coordinates (process/fit/fit.py:38-124,
    non-robust path): scipy curve_fit from a zero start."""
    shape = data.shape
    x, y = np.linspace(0, 1, shape[0]), np.linspace(0, 1, shape[1])
    ry, rx = np.meshgrid(y, x)
    rx_1d = rx.reshape((1, np.prod(shape)))
    ry_1d = ry.reshape((1, np.prod(shape)))
    xy = np.vstack((rx_1d, ry_1d))
    popt = np.zeros((1, len(signature(function).parameters) - 1))
    m1d = mask.reshape((1, np.prod(shape)))
    popt, _ = curve_fit(function, np.vstack((rx_1d[m1d], ry_1d[m1d])), data[mask], p0=popt)
    return function(xy, *popt).reshape(shape)


def fit_origin_surface(com_x, com_y, fit_function="plane", mask=None):
    """Fitted diffraction origin (calibration/origin.py:76-190, default options)."""
    if fit_function == "constant":
        return (np.mean(com_x) * np.ones_like(com_x), np.mean(com_y) * np.ones_like(com_y))
    if fit_function not in _FIT_FUNCTIONS:
        raise ValueError(f"fit_function must be one of {list(_FIT_FUNCTIONS)} or 'constant'")
    f = _FIT_FUNCTIONS[fit_function]
    if mask is None:
        mask = np.ones(com_x.shape, dtype=bool)
    return _fit_surface(f, com_x, mask), _fit_surface(f, com_y, mask)


def rotate_positions(positions, angle):
    """Rotate (J,2) positions about their mean by `angle` (radians), using the
    float32 rotation matrix of the reference's affine helper (utils.py:595-733)."""
    cosx = np.cos(angle)
    sinx = np.sin(angle)
    scale = np.array([[1.0, 0.0], [0.0, 1.0]], dtype="float32")
    shear = np.array([[1.0, 0.0], [0.0, 1.0]], dtype="float32")
    rot = np.array([[+cosx, -sinx], [+sinx, +cosx]], dtype="float32")
    matrix = (scale @ shear @ rot).astype(np.float32)
    origin = np.asarray(positions.mean(0), dtype=np.float32)
    translation = np.array((0.0, 0.0)) + origin
    return ((positions - origin) @ matrix) + translation


# ------------------------------------------------------------------ the mixin


class PreprocessMixin:
    """Preprocessing steps; expects the attributes set by the class constructors."""

    # -- datacube --------------------------------------------------------------
    def _prepare_datacube(self, datacube, diffraction_intensities_shape, reshaping_method,
                          padded_diffraction_intensities_shape, vacuum_probe_intensity,
                          dp_mask, com_shifts, com_measured):
        data = np.asarray(datacube.data)
        rshape = data.shape[:2]
        if com_shifts is not None and np.isscalar(com_shifts[0]):
            com_shifts = (np.ones(rshape) * com_shifts[0], np.ones(rshape) * com_shifts[1])
        if com_measured is not None and np.isscalar(com_measured[0]):
            com_measured = (np.ones(rshape) * com_measured[0], np.ones(rshape) * com_measured[1])

        if diffraction_intensities_shape is not None:
            qx, qy = data.shape[-2:]
            sx, sy = diffraction_intensities_shape
            factor_x, factor_y = sx / qx, sy / qy
            if factor_x != factor_y:
                raise ValueError("Datacube calibration can only handle uniform Q-sampling.")
            if reshaping_method not in ("bin", "fourier", "bilinear"):
                raise ValueError(
                    "reshaping_method needs to be one of 'bilinear', 'fourier', or 'bin', "
                    f"not {reshaping_method}.")
            if com_shifts is not None:
                com_shifts = (com_shifts[0] * factor_x, com_shifts[1] * factor_x)
            if com_measured is not None:
                com_measured = (com_measured[0] * factor_x, com_measured[1] * factor_x)
            q0 = datacube.calibration.get_Q_pixel_size()
            if reshaping_method == "bin":
                binf = int(1 / factor_x)
                if binf < 1:
                    raise ValueError(f"Calculated binning factor {binf} is less than 1.")
                nx, ny = qx // binf, qy // binf
                data = data[..., : nx * binf, : ny * binf].reshape(
                    rshape + (nx, binf, ny, binf)).sum(axis=(-3, -1))
                datacube = _RebinnedCube(data, datacube.calibration, q0 * binf)
                if vacuum_probe_intensity is not None:
                    v = vacuum_probe_intensity[: nx * binf, : ny * binf]
                    vacuum_probe_intensity = v.reshape(nx, binf, ny, binf).sum(axis=(1, 3))
                if dp_mask is not None:
                    v = dp_mask[: nx * binf, : ny * binf]
                    dp_mask = v.reshape(nx, binf, ny, binf).sum(axis=(1, 3))
            elif reshaping_method == "fourier":
                # preprocess/preprocess.py:636-663 (scale given, sums not rescaled)
                out = (np.asarray((qx, qy)) * np.asarray(factor_x)).astype("intp")
                data = fourier_resample(data, tuple(out))
                datacube = _RebinnedCube(data, datacube.calibration, q0 / factor_x)
                if vacuum_probe_intensity is not None:
                    vacuum_probe_intensity = fourier_resample(
                        vacuum_probe_intensity, (sx, sy), force_nonnegative=True)
                if dp_mask is not None:
                    dp_mask = fourier_resample(dp_mask, (sx, sy), force_nonnegative=True,
                                               conserve_array_sums=False)
            else:
                # preprocess/preprocess.py:665-717: per-pattern linear zoom into a
                # float64 cube, divided by the area factor
                from scipy.ndimage import zoom

                f = np.tile(np.asarray(factor_x), 2)
                out = np.round(f * np.array((qx, qy))).astype("int")
                resized = np.zeros(rshape + tuple(out))
                for rx in range(rshape[0]):
                    for ry in range(rshape[1]):
                        resized[rx, ry] = zoom(np.asarray(data[rx, ry], dtype=np.float32), f,
                                               order=1, mode="nearest", grid_mode=True)
                data = resized / f.prod()
                datacube = _RebinnedCube(data, datacube.calibration, q0 / f[0])
                if vacuum_probe_intensity is not None:
                    vacuum_probe_intensity = zoom(vacuum_probe_intensity, (factor_x, factor_x),
                                                  order=1, mode="grid-wrap", grid_mode=True)
                    vacuum_probe_intensity = vacuum_probe_intensity / factor_x ** 2
                if dp_mask is not None:
                    dp_mask = zoom(dp_mask, (factor_x, factor_x), order=1, mode="grid-wrap",
                                   grid_mode=True)

        if padded_diffraction_intensities_shape is not None:
            qx, qy = data.shape[-2:]
            sx, sy = padded_diffraction_intensities_shape
            pad_kx = ((sx - qx) // 2, (sx - qx) // 2 + (sx - qx) % 2)
            pad_ky = ((sy - qy) // 2, (sy - qy) // 2 + (sy - qy) % 2)
            data = np.pad(data, ((0, 0), (0, 0), pad_kx, pad_ky), mode="constant")
            datacube = _RebinnedCube(data, datacube.calibration,
                                     datacube.calibration.get_Q_pixel_size())
            if vacuum_probe_intensity is not None:
                vacuum_probe_intensity = np.pad(vacuum_probe_intensity,
                                                pad_width=(pad_kx, pad_ky), mode="constant")
            if dp_mask is not None:
                dp_mask = np.pad(dp_mask, pad_width=(pad_kx, pad_ky), mode="constant")
        return datacube, vacuum_probe_intensity, dp_mask, com_shifts, com_measured

    def _intensities_and_calibrations(self, datacube, force_scan_sampling,
                                      force_angular_sampling, force_reciprocal_sampling):
        energy = self._energy
        intensities = np.asarray(datacube.data, dtype=np.float32)
        self._grid_scan_shape = intensities.shape[:2]
        cal = datacube.calibration
        r_units = cal.get_R_pixel_units()
        q_units = cal.get_Q_pixel_units()

        if force_scan_sampling is not None:
            self._scan_sampling = (force_scan_sampling, force_scan_sampling)
            self._scan_units = ("A",) * 2
        elif r_units == "A":
            self._scan_sampling = (cal.get_R_pixel_size(),) * 2
            self._scan_units = ("A",) * 2
        elif r_units == "nm":
            self._scan_sampling = (cal.get_R_pixel_size() * 10,) * 2
            self._scan_units = ("A",) * 2
        elif r_units == "pixels":
            raise ValueError("Real-space calibrations must be given in 'A'")
        else:
            raise ValueError(f"Real-space calibrations must be given in 'A', not {r_units}")

        lam = electron_wavelength_angstrom(energy)
        if force_angular_sampling is not None or force_reciprocal_sampling is not None:
            if force_angular_sampling is not None and force_reciprocal_sampling is not None:
                raise ValueError("Only one of angular or reciprocal calibration can be forced.")
            if force_angular_sampling is not None:
                self._angular_sampling = (force_angular_sampling,) * 2
                self._angular_units = ("mrad",) * 2
                self._reciprocal_sampling = (force_angular_sampling / lam / 1e3,) * 2
                self._reciprocal_units = ("A^-1",) * 2
            else:
                self._reciprocal_sampling = (force_reciprocal_sampling,) * 2
                self._reciprocal_units = ("A^-1",) * 2
                self._angular_sampling = (force_reciprocal_sampling * lam * 1e3,) * 2
                self._angular_units = ("mrad",) * 2
        elif q_units == "A^-1":
            size = cal.get_Q_pixel_size()
            self._reciprocal_sampling = (size,) * 2
            self._reciprocal_units = ("A^-1",) * 2
            self._angular_sampling = (size * lam * 1e3,) * 2
            self._angular_units = ("mrad",) * 2
        elif q_units == "mrad":
            size = cal.get_Q_pixel_size()
            self._angular_sampling = (size,) * 2
            self._angular_units = ("mrad",) * 2
            self._reciprocal_sampling = (size / lam / 1e3,) * 2
            self._reciprocal_units = ("A^-1",) * 2
        elif q_units == "pixels":
            raise ValueError("Reciprocal-space calibrations must be given in in 'A^-1' or 'mrad'")
        else:
            raise ValueError(
                f"Reciprocal-space calibrations must be given in 'A^-1' or 'mrad', not {q_units}")
        return intensities

    # -- centre of mass --------------------------------------------------------
    def _intensities_center_of_mass(self, intensities, dp_mask, fit_function, com_shifts,
                                    com_measured, vectorized, intensities_dev=None):
        rs = self._reciprocal_sampling
        if com_measured:
            cmx = np.asarray(com_measured[0], dtype=np.float32)
            cmy = np.asarray(com_measured[1], dtype=np.float32)
        else:
            if dp_mask is not None and dp_mask.shape != intensities.shape[-2:]:
                raise ValueError(
                    f"Mask shape should be (Qx,Qy):{intensities.shape[-2:]}, not {dp_mask.shape}")
            kx = np.arange(intensities.shape[-2], dtype=np.float32)
            ky = np.arange(intensities.shape[-1], dtype=np.float32)
            kya, kxa = np.meshgrid(ky, kx)
            if intensities_dev is not None:
                # the bits of the branch below that `vectorized` selects
                from . import device_preprocess

                cx, cy = device_preprocess.pattern_com(intensities_dev, dp_mask, vectorized)
                cmx = cx.reshape(intensities.shape[:2])
                cmy = cy.reshape(intensities.shape[:2])
            elif vectorized:
                im = intensities * dp_mask if dp_mask is not None else intensities
                isum = np.sum(im, axis=(-2, -1))
                cmx = np.sum(im * kxa[None, None], axis=(-2, -1)) / isum
                cmy = np.sum(im * kya[None, None], axis=(-2, -1)) / isum
            else:
                sx, sy = intensities.shape[:2]
                cmx = np.zeros((sx, sy), dtype=np.float32)
                cmy = np.zeros((sx, sy), dtype=np.float32)
                for rx in range(sx):
                    for ry in range(sy):
                        mi = np.array(intensities[rx, ry])
                        if dp_mask is not None:
                            mi *= dp_mask
                        s = mi.sum()
                        cmx[rx, ry] = np.sum(mi * kxa) / s
                        cmy[rx, ry] = np.sum(mi * kya) / s

        if com_shifts is None:
            if fit_function is not None:
                finite = np.isfinite(np.asarray(cmx))
                fx, fy = fit_origin_surface(np.asarray(cmx), np.asarray(cmy), fit_function, finite)
                cfx = np.asarray(fx, dtype=np.float32)
                cfy = np.asarray(fy, dtype=np.float32)
            else:
                cfx = np.asarray(cmx, dtype=np.float32)
                cfy = np.asarray(cmy, dtype=np.float32)
        else:
            cfx = np.asarray(com_shifts[0], dtype=np.float32)
            cfy = np.asarray(com_shifts[1], dtype=np.float32)

        cnx = np.nan_to_num(cmx - cfx) * rs[0]
        cny = np.nan_to_num(cmy - cfy) * rs[1]
        return cmx, cmy, cfx, cfy, cnx, cny

    # -- rotation --------------------------------------------------------------
    @staticmethod
    def _curl_or_div(cx, cy, maximize_divergence, axis=None):
        if maximize_divergence:
            gxx = cx[..., 2:, 1:-1] - cx[..., :-2, 1:-1]
            gyy = cy[..., 1:-1, 2:] - cy[..., 1:-1, :-2]
            return np.mean(np.abs(gxx + gyy), axis=axis)
        gxy = cx[..., 1:-1, 2:] - cx[..., 1:-1, :-2]
        gyx = cy[..., 2:, 1:-1] - cy[..., :-2, 1:-1]
        return np.mean(np.abs(gyx - gxy), axis=axis)

    @staticmethod
    def _rotated(nx, ny, angle, transpose):
        if transpose:
            return (np.cos(angle) * ny - np.sin(angle) * nx,
                    np.sin(angle) * ny + np.cos(angle) * nx)
        return (np.cos(angle) * nx - np.sin(angle) * ny,
                np.sin(angle) * nx + np.cos(angle) * ny)

    def _rotation_values(self, cnx, cny, rad, maximize_divergence):
        """Mean |curl| (|div|) of the CoM field rotated by each angle of rad
        (A,1,1), untransposed and transposed: two (A,) float32 arrays."""
        if self._device == "gpu":
            from . import device_preprocess

            vals = device_preprocess.rotation_values(
                np.asarray(cnx), np.asarray(cny), np.cos(rad), np.sin(rad), maximize_divergence)
            return vals[0], vals[1]
        return tuple(self._curl_or_div(*self._rotated(cnx[None], cny[None], rad, t),
                                       maximize_divergence, axis=(-2, -1)) for t in (False, True))

    def _solve_rotation(self, cnx, cny, rotation_angles_deg, maximize_divergence,
                        force_com_rotation, force_com_transpose):
        verbose = self._verbose
        if rotation_angles_deg is None:
            rotation_angles_deg = np.arange(-89.0, 90.0, 1.0)

        def better(a, b):  # is the transposed value a better than b?
            return a > b if maximize_divergence else a < b

        if force_com_rotation is not None:
            best_rad = np.deg2rad(force_com_rotation)
            if verbose:
                warnings.warn(f"Best fit rotation forced to {force_com_rotation:.0f} degrees.",
                              UserWarning)
            if force_com_transpose is not None:
                best_t = force_com_transpose
                if verbose:
                    warnings.warn(f"Transpose of intensities forced to {force_com_transpose}.",
                                  UserWarning)
            else:
                v0 = self._curl_or_div(*self._rotated(cnx, cny, best_rad, False),
                                       maximize_divergence)
                v1 = self._curl_or_div(*self._rotated(cnx, cny, best_rad, True),
                                       maximize_divergence)
                best_t = better(v1, v0)
                if verbose and best_t:
                    warnings.warn("Diffraction intensities should be transposed.", UserWarning)
        else:
            deg = np.asarray(rotation_angles_deg, dtype=np.float32)
            rad = np.deg2rad(deg)[:, None, None]
            pick = np.argmax if maximize_divergence else np.argmin
            rad_flat = np.squeeze(rad)
            if force_com_transpose is not None:
                best_t = force_com_transpose
                if verbose:
                    warnings.warn(f"Transpose of intensities forced to {force_com_transpose}.",
                                  UserWarning)
                vals = self._rotation_values(cnx, cny, rad, maximize_divergence)[int(best_t)]
                i = pick(vals).item()
                best_deg, best_rad = deg[i], rad_flat[i]
            else:
                v0, v1 = self._rotation_values(cnx, cny, rad, maximize_divergence)
                i0 = pick(v0).item()
                i1 = pick(v1).item()
                keep0 = v0[i0] >= v1[i1] if maximize_divergence else v0[i0] <= v1[i1]
                if keep0:
                    best_deg, best_rad, best_t = deg[i0], rad_flat[i0], False
                else:
                    best_deg, best_rad, best_t = deg[i1], rad_flat[i1], True
                self._rotation_angles_deg = deg
            if verbose:
                warnings.warn(f"Best fit rotation = {best_deg:.0f} degrees.", UserWarning)
                if best_t and force_com_transpose is None:
                    warnings.warn("Diffraction intensities should be transposed.", UserWarning)
        com_x, com_y = self._rotated(cnx, cny, best_rad, best_t)
        return best_rad, best_t, com_x, com_y

    # -- amplitudes ------------------------------------------------------------
    @staticmethod
    def _crop_geometry(pattern_shape, cfx, cfy, crop_patterns):
        """(crop width, crop mask, cropped shape) of the corner crop
        (phase_base_class.py:1385-1400); width 0 and no mask without cropping."""
        if not crop_patterns:
            return 0, None, tuple(pattern_shape)
        crop_x = int(np.minimum(pattern_shape[0] - cfx.max(), cfx.min()))
        crop_y = int(np.minimum(pattern_shape[1] - cfy.max(), cfy.min()))
        w = int(np.minimum(crop_y, crop_x))
        crop_mask = np.zeros(pattern_shape, dtype="bool")
        crop_mask[:w, :w] = True
        crop_mask[-w:, :w] = True
        crop_mask[:w:, -w:] = True
        crop_mask[-w:, -w:] = True
        return w, crop_mask, (w * 2, w * 2)

    def _normalize_intensities_device(self, intensities_dev, com_fitted_x, com_fitted_y,
                                      positions_mask, crop_patterns):
        """Device amplitudes, float32 mean intensity, crop mask and shape; the
        same values as _normalize_intensities (the caller's datacube is left
        unmodified)."""
        from . import device_preprocess

        cfx = np.asarray(com_fitted_x)
        cfy = np.asarray(com_fitted_y)
        w, crop_mask, crop_shape = self._crop_geometry(tuple(intensities_dev.shape[-2:]), cfx,
                                                       cfy, crop_patterns)
        if crop_patterns and (w < 1 or 2 * w > min(intensities_dev.shape[-2:])):
            raise NotImplementedError(
                f"corner crop of width {w} on {tuple(intensities_dev.shape[-2:])} patterns")
        amps, mean = device_preprocess.normalize_patterns(intensities_dev, cfx, cfy,
                                                          positions_mask, w)
        return amps, mean, crop_mask, crop_shape

    def _normalize_intensities(self, intensities, com_fitted_x, com_fitted_y,
                               positions_mask, crop_patterns, in_place):
        diff = intensities if in_place else intensities.copy()
        cfx = np.asarray(com_fitted_x)
        cfy = np.asarray(com_fitted_y)
        _, crop_mask, crop_shape = self._crop_geometry(diff.shape[-2:], cfx, cfy, crop_patterns)

        # mean intensity accumulates in float32 pattern by pattern, like the reference
        mean_intensity = 0
        for rx in range(diff.shape[0]):
            for ry in range(diff.shape[1]):
                if positions_mask is not None and not positions_mask[rx, ry]:
                    continue
                shifted = shift_bilinear(diff[rx, ry], -cfx[rx, ry], -cfy[rx, ry])
                mean_intensity += np.sum(shifted)
                diff[rx, ry] = np.sqrt(np.maximum(shifted, 0))

        if positions_mask is not None:
            diff = diff[positions_mask]
        else:
            qx, qy = diff.shape[-2:]
            diff = diff.reshape((-1, qx, qy))
        if crop_patterns:
            diff = diff[:, crop_mask].reshape((-1,) + crop_shape)
        mean_intensity /= diff.shape[0]
        return diff, mean_intensity, crop_mask, crop_shape

    # -- positions -------------------------------------------------------------
    def _scan_positions_in_pixels(self, positions, positions_mask, object_padding_px,
                                  positions_offset_ang):
        sampling = self.sampling
        if positions is None:
            nx, ny = self._grid_scan_shape
            sx, sy = self._scan_sampling
            x = np.arange(nx) * sx
            y = np.arange(ny) * sy
            x, y = np.meshgrid(x, y, indexing="ij")
            if positions_offset_ang is not None:
                x += positions_offset_ang[0]
                y += positions_offset_ang[1]
            if positions_mask is not None:
                x = x[positions_mask]
                y = y[positions_mask]
            positions = np.stack((x.ravel(), y.ravel()), axis=-1)
        else:
            positions = np.array(positions, copy=True)
        if self._rotation_best_rad is not None:
            positions = rotate_positions(positions, self._rotation_best_rad)
        if self._rotation_best_transpose:
            positions = np.flip(positions, 1)
            sampling = sampling[::-1]
        positions -= np.min(positions, axis=0).clip(-np.inf, 0)
        positions[:, 0] /= sampling[0]
        positions[:, 1] /= sampling[1]
        roi = self._region_of_interest_shape
        if object_padding_px is None:
            pad = roi / 2
            object_padding_px = (pad, pad)
        elif np.isscalar(object_padding_px[0]):
            object_padding_px = ((object_padding_px[0],) * 2, (object_padding_px[1],) * 2)
        positions[:, 0] += object_padding_px[0][0]
        positions[:, 1] += object_padding_px[1][0]
        return positions, object_padding_px

    # -- object ----------------------------------------------------------------
    def _object_extent(self, positions_px):
        roi = self._region_of_interest_shape
        if self._object_fov_ang is None:
            pad_x = self._object_padding_px[0][1]
            pad_y = self._object_padding_px[1][1]
            p, q = np.round(np.max(positions_px, axis=0))
            p = np.max([np.round(p + pad_x), roi[0]]).astype("int")
            q = np.max([np.round(q + pad_y), roi[1]]).astype("int")
        else:
            p, q = np.ceil(np.array(self._object_fov_ang) / np.array(self.sampling)).astype("int")
        return int(p), int(q)

    def _initial_object(self, initial_object, positions_px, object_type, num_slices=None):
        if initial_object is None:
            p, q = self._object_extent(positions_px)
            shape = (p, q) if num_slices is None else (num_slices, p, q)
            if object_type == "potential":
                return np.zeros(shape, dtype=np.float32)
            return np.ones(shape, dtype=np.complex64)
        if object_type == "potential":
            return np.asarray(initial_object, dtype=np.float32)
        return np.asarray(initial_object, dtype=np.complex64)

    # -- probe -----------------------------------------------------------------
    def _single_probe(self, initial_probe, vacuum_probe_intensity, mean_intensity,
                      semiangle_cutoff, crop_patterns):
        roi = self._region_of_interest_shape
        if initial_probe is None:
            if vacuum_probe_intensity is not None:
                semiangle_cutoff = np.inf
                vpi = np.asarray(vacuum_probe_intensity, dtype=np.float32)
                x0, y0 = center_of_mass(vpi)
                vpi = shift_bilinear(vpi, -x0, -y0)
                if crop_patterns:
                    vpi = vpi[self._crop_mask].reshape(self._crop_mask_shape)
                sx, sy = vpi.shape
                tx, ty = (int(v) for v in roi)
                # the reference's condition as written (ptychographic_methods.py:1056-1064:
                # `or` binds the x test alone)
                if sx != tx or sy != ty and self._resample_exit_waves is True:
                    vpi = bilinear_resample(vpi, (tx, ty), conserve_array_sums=True)
                vacuum_probe_intensity = vpi
            probe = ComplexProbe(
                gpts=roi, sampling=self.sampling, energy=self._energy,
                semiangle_cutoff=semiangle_cutoff, rolloff=self._rolloff,
                vacuum_probe_intensity=vacuum_probe_intensity,
                parameters=self._polar_parameters).build()._array
            intensity = np.sum(np.abs(np.fft.fft2(probe)) ** 2)
            probe *= np.sqrt(mean_intensity / intensity)
        elif isinstance(initial_probe, ComplexProbe):
            if tuple(initial_probe._gpts) != tuple(roi):
                raise ValueError("initial ComplexProbe gpts do not match the ROI shape")
            probe = initial_probe._array if hasattr(initial_probe, "_array") else \
                initial_probe.build()._array
            intensity = np.sum(np.abs(np.fft.fft2(probe)) ** 2)
            probe *= np.sqrt(mean_intensity / intensity)
        else:
            probe = np.asarray(initial_probe, dtype=np.complex64)
        return probe, semiangle_cutoff

    def _mixed_probes(self, initial_probe, vacuum_probe_intensity, mean_intensity,
                      semiangle_cutoff, crop_patterns):
        """Mode 0 is the single probe; each further mode is the previous one times
        random linear phase ramps drawn from NumPy's global RNG
        (ptychographic_methods.py:1416-1462)."""
        if initial_probe is None or isinstance(initial_probe, ComplexProbe):
            probe, semiangle_cutoff = self._single_probe(
                initial_probe, vacuum_probe_intensity, mean_intensity, semiangle_cutoff,
                crop_patterns)
            sx, sy = self._region_of_interest_shape
            probes = np.zeros((self._num_probes, sx, sy), dtype=np.complex64)
            probes[0] = probe
            for i in range(1, self._num_probes):
                shift_x = np.exp(-2j * np.pi * (np.random.rand() - 0.5) * np.fft.fftfreq(sx))
                shift_y = np.exp(-2j * np.pi * (np.random.rand() - 0.5) * np.fft.fftfreq(sy))
                probes[i] = probes[i - 1] * shift_x[:, None] * shift_y[None]
            return probes, semiangle_cutoff
        return np.asarray(initial_probe, dtype=np.complex64), semiangle_cutoff

    # -- overlap / FOV mask ----------------------------------------------------
    @staticmethod
    def _fourier_shift(array, positions):
        """ifft2(fft2(array) x exp(-2 pi i (kx x + ky y))) for (B,2) positions
        (utils.py:468-533), complex64 arithmetic."""
        sx, sy = array.shape[-2:]
        kx = np.fft.fftfreq(sx, 1.0).astype(np.float32)
        ky = np.fft.fftfreq(sy, 1.0).astype(np.float32)
        pos = np.asarray(positions, dtype=np.float32)
        single = pos.ndim == 1
        if single:
            pos = pos[None]
        x = pos[:, 0].ravel()[:, None, None]
        y = pos[:, 1].ravel()[:, None, None]
        op = np.exp(-2.0j * np.pi * kx[None, :, None] * x) * np.exp(
            -2.0j * np.pi * ky[None, None, :] * y)
        if single:
            op = op[0]
        fa = np.fft.fft2(array)
        if op.ndim == 3 and fa.ndim == 3:
            shifted = fa[None] * op[:, None]
        else:
            shifted = fa * op
        return np.fft.ifft2(shifted)

    def _scatter_patches(self, patches, positions_px):
        """Sum (B,Sx,Sy) real patches into the object grid with periodic wrap,
        float64 accumulation then float32 (phase_base_class.py:1905-1940)."""
        roi = self._region_of_interest_shape
        shape = self._object_shape
        x0 = np.round(positions_px[:, 0]).astype("int")
        y0 = np.round(positions_px[:, 1]).astype("int")
        xi = np.fft.fftfreq(roi[0], d=1 / roi[0]).astype("int")
        yi = np.fft.fftfreq(roi[1], d=1 / roi[1]).astype("int")
        idx = ((y0[:, None, None] + yi[None, None, :]) % shape[1]) + (
            (x0[:, None, None] + xi[None, :, None]) % shape[0]) * shape[1]
        counts = np.bincount(idx.ravel(), weights=patches.ravel(),
                             minlength=int(np.prod(shape)))
        return np.reshape(counts, shape).astype(np.float32)

    def _probe_overlap(self, probe_single, max_batch_size):
        if self._device == "gpu":
            from . import device_preprocess

            return device_preprocess.probe_overlap(probe_single, self._positions_px,
                                                   self._object_shape, max_batch_size)
        if max_batch_size is None:
            max_batch_size = self._num_diffraction_patterns
        overlap = np.zeros(self._object_shape, dtype=np.float32)
        for start, end in generate_batches(self._num_diffraction_patterns, max_batch_size):
            pos = self._positions_px[start:end]
            frac = pos - np.round(pos)
            shifted = self._fourier_shift(probe_single, frac)
            overlap += self._scatter_patches(np.abs(shifted) ** 2, pos)
        return overlap

    def _fov_mask(self, object_fov_mask, probe_overlap):
        if object_fov_mask is None:
            blurred = gaussian_filter(probe_overlap, 1.0)
            mask = np.asarray(blurred > 0.25 * blurred.max())
        elif object_fov_mask is True:
            mask = np.full(self._object_shape, True)
        else:
            mask = np.asarray(object_fov_mask)
        return mask


class _RebinnedCube:
    """Datacube view after binning or padding in preprocess."""

    def __init__(self, data, calibration, q_pixel_size):
        self.data = data
        self._cal = calibration
        self._q = q_pixel_size

        class _Cal:
            def get_R_pixel_size(_s):
                return calibration.get_R_pixel_size()

            def get_R_pixel_units(_s):
                return calibration.get_R_pixel_units()

            def get_Q_pixel_size(_s):
                return q_pixel_size

            def get_Q_pixel_units(_s):
                return calibration.get_Q_pixel_units()

        self.calibration = _Cal()

    @property
    def shape(self):
        return self.data.shape

    @property
    def Rshape(self):
        return self.data.shape[:2]
