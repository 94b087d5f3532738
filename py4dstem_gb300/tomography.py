"""Ptychographic tomography on the GPU: the multislice position loop of every
tilt, run on the slices of a rotated 3D potential volume.

Drop-in for ``PtychographicTomography`` of py4DSTEM 0.14.18
(process/phase/ptychographic_tomography.py): same constructor, ``preprocess()``
and ``reconstruct()`` arguments, same state and results (``object`` the
(Z, Px, Py) volume, ``probe`` one centred probe per tilt, ``error_iterations``).

Per iteration, for each tilt in a shuffled order (ptychographic_tomography.py:
974-1240), everything on the device:

* the volume is rotated into the tilt's frame (``ptycho_volume_rotate``: cubic
  B-spline resampling, float64, as scipy.ndimage.affine_transform);
* it is summed onto the multislice slices (``ptycho_volume_project``);
* the tilt's batches run through the fused multislice gradient-descent kernels
  on those slices with the tilt's probe, positions and amplitudes (the same
  kernels as ``MultislicePtychography`` with a potential object);
* the slice update is spread back over the voxels
  (``ptycho_volume_expand_update``) and, with collective updates (the default),
  rotated back and summed for one volume update at the end of the iteration;
  otherwise added to the volume at once.

What the reference computes and throws away is not computed: its per-tilt probe
constraints return a new probe into a local name that is never stored
(ptychographic_tomography.py:1139-1161), so the per-tilt probes carry the
gradient updates only, here as there. The volume's 3D Gaussian blur runs among
the object constraints (the object Gaussian kernels over the volume's Z
slices). Not implemented (they raise): projection sets and position correction,
which the reference's own tomography loop cannot run either (with projection
sets its _forward call fails, "can't multiply sequence by non-int of type
'float'", ptychographic_tomography.py:1065; position correction passes the
forward's per-slice probe stack where the slice-0 probe is expected and fails
to broadcast, :1097 into ptychographic_methods.py:2342), the 3D Butterworth
filter (an FFT of the whole volume) and TV denoising (pylops).
"""

from __future__ import annotations

import ctypes
import dataclasses
import warnings
from typing import Mapping, Sequence, Tuple

import numpy as np

from . import _native, engine
from .ptychography import _PtychographyBase, method_parameters

_SWAP_ZXY_TO_XYZ = np.array([[0, 1, 0], [0, 0, 1], [1, 0, 0]])


def rotation_transform(shape, rot_matrix):
    """(matrix, offset) that _rotate_zxy_volume hands to affine_transform for a
    volume of `shape` (ptychographic_methods.py:849-868), in float64."""
    tf = _SWAP_ZXY_TO_XYZ.T @ np.asarray(rot_matrix).T @ _SWAP_ZXY_TO_XYZ
    in_center = (np.asarray(shape) - 1) / 2
    out_center = tf @ in_center
    return np.ascontiguousarray(tf, dtype=np.float64), np.ascontiguousarray(
        in_center - out_center, dtype=np.float64)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class VolumeOps:
    """Device buffers and calls of the volume operations for one volume shape."""

    def __init__(self, shape, num_slices, device):
        torch = engine._torch()
        self.shape = tuple(int(v) for v in shape)
        self.T = int(num_slices)
        n = int(np.prod(self.shape))
        self.scratch = torch.empty(n, dtype=torch.float64, device=device)
        self.update = torch.empty(n, dtype=torch.float64, device=device)
        self.lib = _native.lib()
        self.launches = 0

    def _stream(self):
        return ctypes.c_void_p(engine._torch().cuda.current_stream().cuda_stream)

    def rotate(self, src, dst, rot_matrix, out_mode):
        """dst = src rotated by rot_matrix; out_mode 0 float32, 1 float64, 2 add into float32."""
        tf, off = rotation_transform(self.shape, rot_matrix)
        n0, n1, n2 = self.shape
        _native.check(self.lib.ptycho_volume_rotate(
            _ptr(src), 1 if src.dtype == engine._torch().float64 else 0, _ptr(dst), out_mode,
            n0, n1, n2, tf.ctypes.data_as(ctypes.c_void_p), off.ctypes.data_as(ctypes.c_void_p),
            _ptr(self.scratch), ctypes.c_size_t(self.scratch.numel() * 8), self._stream()))
        self.launches += 2 + sum(1 for v in self.shape if v > 1)

    def project(self, volume, sliced):
        n0, n1, n2 = self.shape
        _native.check(self.lib.ptycho_volume_project(_ptr(volume), n0, n1, n2, self.T,
                                                     _ptr(sliced), self._stream()))
        self.launches += 1

    def expand(self, sliced, sliced_old, out, out_mode):
        n0, n1, n2 = self.shape
        _native.check(self.lib.ptycho_volume_expand_update(
            _ptr(sliced), _ptr(sliced_old), self.T, n0, n1, n2, _ptr(out), out_mode,
            self._stream()))
        self.launches += 1

    def add_scaled(self, volume, addend, divisor):
        _native.check(self.lib.ptycho_volume_add_scaled(
            _ptr(volume), _ptr(addend), ctypes.c_int64(volume.numel()), int(divisor),
            self._stream()))
        self.launches += 1

    def gaussian(self, volume, sigma_px, roi):
        """scipy.ndimage.gaussian_filter of the whole (Z, Px, Py) volume, every axis
        (ptychographic_constraints.py:119-151 as the 3D object constraints call it,
        :836-887): the object Gaussian kernels of the reconstruction over the
        volume taken as Z slices."""
        torch = engine._torch()
        radius = int(4.0 * sigma_px + 0.5)
        x = np.arange(-radius, radius + 1)
        phi = np.exp(-0.5 / (sigma_px * sigma_px) * x ** 2)
        w = torch.from_numpy(np.ascontiguousarray(phi / phi.sum())).to(volume.device)
        if getattr(self, "gauss_scratch", None) is None:
            self.gauss_scratch = torch.empty(4 * volume.numel(), dtype=torch.float32,
                                             device=volume.device)
        n0, n1, n2 = self.shape
        g = _native.Geometry(int(roi[0]), int(roi[1]), n1, n2, n0, 1, 1, 0)
        _native.check(self.lib.ptycho_object_gaussian_constraint(
            ctypes.byref(g), _ptr(volume), _ptr(w), radius, 0, _ptr(self.gauss_scratch),
            self._stream()))
        self.launches += 3 if n0 > 1 else 2

    def constraints(self, volume, shrinkage_rad, positivity):
        shrink = shrinkage_rad > 0.0
        if not shrink and not positivity:
            return
        _native.check(self.lib.ptycho_volume_constraints(
            _ptr(volume), ctypes.c_int64(volume.numel()), ctypes.c_float(shrinkage_rad),
            1 if shrink else 0, 1 if positivity else 0, self._stream()))
        self.launches += 1


class PtychographicTomography(_PtychographyBase):
    """Joint ptychographic tomography of a (Z, Px, Py) potential volume."""

    _multislice = True

    def __init__(
        self,
        energy: float,
        num_slices: int,
        tilt_orientation_matrices: Sequence[np.ndarray],
        datacube=None,
        semiangle_cutoff: float = None,
        semiangle_cutoff_pixels: float = None,
        rolloff: float = 2.0,
        vacuum_probe_intensity: np.ndarray = None,
        polar_parameters: Mapping[str, float] = None,
        object_padding_px: Tuple[int, int] = None,
        object_type: str = "potential",
        positions_mask: np.ndarray = None,
        initial_object_guess: np.ndarray = None,
        initial_probe_guess: np.ndarray = None,
        initial_scan_positions: Sequence[np.ndarray] = None,
        positions_offset_ang: Sequence[np.ndarray] = None,
        verbose: bool = True,
        device: str = "gpu",
        storage: str = None,
        clear_fft_cache: bool = True,
        name: str = "ptychographic-tomography_reconstruction",
        **kwargs,
    ):
        num_tilts = len(tilt_orientation_matrices)
        if initial_scan_positions is None:
            initial_scan_positions = [None] * num_tilts
        if object_type != "potential":
            raise NotImplementedError()
        self._common_init(energy, datacube, semiangle_cutoff, semiangle_cutoff_pixels, rolloff,
                          vacuum_probe_intensity, polar_parameters, initial_object_guess,
                          initial_probe_guess, initial_scan_positions, None,
                          positions_offset_ang, object_padding_px, object_type, positions_mask,
                          verbose, device, storage, clear_fft_cache, name, kwargs)
        self._probe_init = initial_probe_guess
        self._probe = None
        self._num_slices = num_slices
        self._theta_x = None
        self._theta_y = None
        self._tilt_orientation_matrices = tuple(tilt_orientation_matrices)
        self._num_measurements = num_tilts

    # -- preprocess (ptychographic_tomography.py:215-747) ------------------------
    def preprocess(
        self,
        diffraction_intensities_shape: Tuple[int, int] = None,
        reshaping_method: str = "bilinear",
        padded_diffraction_intensities_shape: Tuple[int, int] = None,
        region_of_interest_shape: Tuple[int, int] = None,
        dp_mask: np.ndarray = None,
        in_place_datacube_modification: bool = False,
        fit_function: str = "plane",
        plot_probe_overlaps: bool = True,
        rotation_real_space_degrees: float = None,
        diffraction_patterns_rotate_degrees: float = None,
        diffraction_patterns_transpose: bool = None,
        force_com_shifts: Sequence[float] = None,
        force_com_measured: Sequence[np.ndarray] = None,
        vectorized_com_calculation: bool = True,
        force_scan_sampling: float = None,
        force_angular_sampling: float = None,
        force_reciprocal_sampling: float = None,
        progress_bar: bool = True,
        object_fov_mask: np.ndarray = True,
        crop_patterns: bool = False,
        main_tilt_axis: str = "vertical",
        store_initial_arrays: bool = True,
        device: str = None,
        clear_fft_cache: bool = None,
        max_batch_size: int = None,
        **kwargs,
    ):
        """Per tilt: the datacube's centre of mass, corner-centred amplitudes and
        scan positions (diffraction rotation given, not searched); then the zero
        volume, one probe per tilt and the Fresnel propagators of the slices.
        plot_* and progress_bar are ignored."""
        self.set_device(device, clear_fft_cache)
        self._diffraction_intensities_shape = diffraction_intensities_shape
        self._reshaping_method = reshaping_method
        self._padded_diffraction_intensities_shape = padded_diffraction_intensities_shape
        self._dp_mask = dp_mask
        if self._datacube is None:
            raise ValueError(
                "The preprocess() method requires a DataCube. "
                "Please run ptycho.attach_datacube(DataCube) first.")
        n_meas = self._num_measurements
        if self._positions_mask is not None:
            self._positions_mask = np.asarray(self._positions_mask, dtype="bool")
            if self._positions_mask.ndim == 2:
                warnings.warn("2D `positions_mask` assumed the same for all measurements.",
                              UserWarning)
                self._positions_mask = np.tile(self._positions_mask, (n_meas, 1, 1))
            counts = np.insert(self._positions_mask.sum(axis=(-2, -1)), 0, 0)
        else:
            self._positions_mask = [None] * n_meas
            counts = np.array([0] + [int(np.prod(dc.data.shape[:2])) for dc in self._datacube])
        self._mean_diffraction_intensity = []
        self._num_diffraction_patterns = counts.sum()
        self._cum_probes_per_measurement = np.cumsum(counts)
        self._positions_px_all = np.empty((self._num_diffraction_patterns, 2))

        if force_com_shifts is None:
            force_com_shifts = [None] * n_meas
        else:
            force_com_shifts = list(force_com_shifts)
        if force_com_measured is None:
            force_com_measured = [None] * n_meas
        else:
            force_com_measured = list(force_com_measured)
        if self._positions_offset_ang is None:
            self._positions_offset_ang = [None] * n_meas
        self._rotation_best_rad = np.deg2rad(diffraction_patterns_rotate_degrees)
        self._rotation_best_transpose = diffraction_patterns_transpose
        datacubes = list(self._datacube)

        host_amps, dev_amps = [], []
        for index in range(n_meas):
            first = index == 0
            (datacubes[index], vpi, mask, force_com_shifts[index],
             force_com_measured[index]) = self._prepare_datacube(
                datacubes[index], diffraction_intensities_shape, reshaping_method,
                padded_diffraction_intensities_shape,
                self._vacuum_probe_intensity if first else None,
                self._dp_mask if first else None, force_com_shifts[index],
                force_com_measured[index])
            if first:
                self._vacuum_probe_intensity, self._dp_mask = vpi, mask
            intensities = self._intensities_and_calibrations(
                datacubes[index], force_scan_sampling, force_angular_sampling,
                force_reciprocal_sampling)
            intensities_dev = None
            if self._device == "gpu":
                from . import device_preprocess

                intensities_dev = device_preprocess.upload_intensities(intensities)
            (_, _, com_fitted_x, com_fitted_y, _, _) = self._intensities_center_of_mass(
                intensities, self._dp_mask, fit_function, force_com_shifts[index],
                force_com_measured[index], vectorized_com_calculation, intensities_dev)
            if intensities_dev is not None:
                amps, mean, self._crop_mask, self._crop_mask_shape = \
                    self._normalize_intensities_device(
                        intensities_dev, com_fitted_x, com_fitted_y,
                        self._positions_mask[index], crop_patterns)
                del intensities_dev
                dev_amps.append(amps)
            else:
                amps, mean, self._crop_mask, self._crop_mask_shape = self._normalize_intensities(
                    intensities, com_fitted_x, com_fitted_y, self._positions_mask[index],
                    crop_patterns, in_place_datacube_modification)
                host_amps.append(np.asarray(amps, dtype=np.float32))
            self._mean_diffraction_intensity.append(mean)
            del intensities
            if first:
                amp_shape = tuple((dev_amps or host_amps)[0].shape[-2:])
                self._amplitudes_shape = np.array(amp_shape)
                if region_of_interest_shape is not None and \
                        tuple(region_of_interest_shape) != amp_shape:
                    raise NotImplementedError(
                        "region_of_interest_shape different from the detector shape "
                        "(exit-wave resampling) is not implemented")
                self._resample_exit_waves = False
                self._region_of_interest_shape = np.array(amp_shape)
            start, end = self._cum_probes_per_measurement[index:index + 2]
            (self._positions_px_all[start:end],
             self._object_padding_px) = self._scan_positions_in_pixels(
                self._scan_positions[index], self._positions_mask[index],
                self._object_padding_px, self._positions_offset_ang[index])
        self._datacube = datacubes
        if dev_amps:
            import torch

            self._set_device_amplitudes(torch.cat(dev_amps, dim=0))
        else:
            self._amplitudes = np.concatenate(host_amps, axis=0)

        if self._semiangle_cutoff_pixels:
            self._semiangle_cutoff = self._semiangle_cutoff_pixels * self._angular_sampling[0]

        self._object = self._initial_volume(self._object, self._positions_px_all,
                                            main_tilt_axis)
        if store_initial_arrays:
            self._object_initial = self._object.copy()
            self._object_type_initial = self._object_type
        self._object_shape = self._object.shape[-2:]
        self._num_voxels = self._object.shape[0]

        # scan positions of each tilt centred on the object (float32 state)
        self._positions_px_all = np.asarray(self._positions_px_all, dtype=np.float32)
        for index in range(n_meas):
            start, end = self._cum_probes_per_measurement[index:index + 2]
            positions_px = self._positions_px_all[start:end]
            positions_px_com = positions_px.mean(0)
            positions_px -= positions_px_com - np.array(self._object_shape) / 2
            self._positions_px_all[start:end] = positions_px.copy()
        self._positions_px_initial_all = self._positions_px_all.copy()
        self._positions_initial_all = self._positions_px_initial_all.copy()
        self._positions_initial_all[:, 0] *= self.sampling[0]
        self._positions_initial_all[:, 1] *= self.sampling[1]

        list_q = isinstance(self._probe_init, (list, tuple))
        self._probes_all = []
        self._probes_all_initial = [] if store_initial_arrays else None
        self._probes_all_initial_aperture = [] if store_initial_arrays else [None] * n_meas
        for index in range(n_meas):
            probe, self._semiangle_cutoff = self._single_probe(
                self._probe_init[index] if list_q else self._probe_init,
                self._vacuum_probe_intensity, self._mean_diffraction_intensity[index],
                self._semiangle_cutoff, crop_patterns)
            probe = np.asarray(probe, dtype=np.complex64)
            self._probes_all.append(probe)
            if store_initial_arrays:
                self._probes_all_initial.append(probe.copy())
                self._probes_all_initial_aperture.append(np.abs(np.fft.fft2(probe)))

        if main_tilt_axis == "vertical":
            thickness = self._object_shape[1] * self.sampling[1]
        elif main_tilt_axis == "horizontal":
            thickness = self._object_shape[0] * self.sampling[0]
        else:
            thickness = max(self._object_shape[1] * self.sampling[1],
                            self._object_shape[0] * self.sampling[0])
        self._slice_thicknesses = np.tile(thickness / self._num_slices, self._num_slices - 1)
        self._propagator_arrays = self._fresnel_propagators()

        if object_fov_mask is not True:
            raise NotImplementedError()
        self._object_fov_mask = np.full(self._object_shape, True)
        self._object_fov_mask_inverse = np.invert(self._object_fov_mask)
        self._preprocessed = True
        return self

    def _initial_volume(self, initial_object, positions_px, main_tilt_axis):
        """(q, p, q), (p, p, q) or (max(p, q), p, q) zeros by main_tilt_axis
        (ptychographic_methods.py:870-912)."""
        if initial_object is not None:
            return np.asarray(initial_object, dtype=np.float32)
        p, q = self._object_extent(positions_px)
        if main_tilt_axis == "vertical":
            return np.zeros((q, p, q), dtype=np.float32)
        if main_tilt_axis == "horizontal":
            return np.zeros((p, p, q), dtype=np.float32)
        return np.zeros((max(p, q), p, q), dtype=np.float32)

    # -- state views (ptychographic_methods.py:3464-3572) ------------------------
    @property
    def probe_centered(self):
        if getattr(self, "_probes_all", None) is None:
            return None
        return [np.fft.fftshift(np.asarray(pr, dtype=np.complex64), axes=(-2, -1))
                for pr in self._probes_all]

    @property
    def probe_fourier(self):
        if getattr(self, "_probes_all", None) is None:
            return None
        return [np.fft.fftshift(np.fft.fft2(np.asarray(pr, dtype=np.complex64)), axes=(-2, -1))
                for pr in self._probes_all]

    @property
    def positions(self):
        if self._angular_sampling is None:
            return None
        out = []
        for index in range(self._num_measurements):
            start, end = self._cum_probes_per_measurement[index:index + 2]
            pos = self._positions_px_all[start:end].copy()
            pos[:, 0] *= self.sampling[0]
            pos[:, 1] *= self.sampling[1]
            out.append(pos)
        return np.asarray(out)

    @property
    def object_supersliced(self):
        """The volume summed onto the slices (ptychographic_methods.py:1000-1004)."""
        z = self._object.shape[0]
        vps = int(np.ceil(z / self._num_slices))
        padded = np.pad(self._object, ((0, vps * self._num_slices - z), (0, 0), (0, 0)))
        return np.sum(padded.reshape((-1, vps) + self._object.shape[1:]), axis=1)

    def _return_self_consistency_errors(self, **kwargs):
        raise NotImplementedError()


    def _reset_tomography(self, store_iterations, reset):
        """MultipleMeasurementsMethodsMixin._reset_reconstruction
        (ptychographic_methods.py:3409-3462), gradient descent."""
        if store_iterations and (not hasattr(self, "object_iterations") or reset):
            self.object_iterations = []
            self.probe_iterations = []
        if reset is True:
            self.error_iterations = []
            self._object = self._object_initial.copy()
            self._probes_all = [pr.copy() for pr in self._probes_all_initial]
            self._positions_px_all = self._positions_px_initial_all.copy()
            self._object_type = self._object_type_initial
            self._exit_waves = None
        elif reset is None:
            if hasattr(self, "error"):
                warnings.warn("Continuing reconstruction from previous result. "
                              "Use reset=True for a fresh start.", UserWarning)
            else:
                self.error_iterations = []
                self._exit_waves = None
        elif not hasattr(self, "error"):
            self.error_iterations = []
            self._exit_waves = None

    # -- reconstruct (ptychographic_tomography.py:749-1269) -----------------------
    def reconstruct(
        self,
        num_iter: int = 8,
        reconstruction_method: str = "gradient-descent",
        reconstruction_parameter: float = 1.0,
        reconstruction_parameter_a: float = None,
        reconstruction_parameter_b: float = None,
        reconstruction_parameter_c: float = None,
        max_batch_size: int = None,
        seed_random: int = None,
        step_size: float = 0.5,
        normalization_min: float = 1,
        positions_step_size: float = 0.9,
        fix_probe_com: bool = True,
        fix_probe: bool = False,
        fix_probe_aperture: bool = False,
        constrain_probe_amplitude: bool = False,
        constrain_probe_amplitude_relative_radius: float = 0.5,
        constrain_probe_amplitude_relative_width: float = 0.05,
        constrain_probe_fourier_amplitude: bool = False,
        constrain_probe_fourier_amplitude_max_width_pixels: float = 3.0,
        constrain_probe_fourier_amplitude_constant_intensity: bool = False,
        fix_positions: bool = True,
        fix_positions_com: bool = True,
        max_position_update_distance: float = None,
        max_position_total_distance: float = None,
        global_affine_transformation: bool = False,
        gaussian_filter_sigma: float = None,
        gaussian_filter: bool = True,
        fit_probe_aberrations: bool = False,
        fit_probe_aberrations_max_angular_order: int = 4,
        fit_probe_aberrations_max_radial_order: int = 4,
        fit_probe_aberrations_remove_initial: bool = False,
        fit_probe_aberrations_using_scikit_image: bool = True,
        butterworth_filter: bool = True,
        q_lowpass: float = None,
        q_highpass: float = None,
        butterworth_order: float = 2,
        object_positivity: bool = True,
        shrinkage_rad: float = 0.0,
        fix_potential_baseline: bool = True,
        detector_fourier_mask: np.ndarray = None,
        tv_denoise: bool = True,
        tv_denoise_weights: float = None,
        tv_denoise_inner_iter=40,
        collective_measurement_updates: bool = True,
        store_iterations: bool = False,
        progress_bar: bool = True,
        reset: bool = None,
        device: str = None,
        clear_fft_cache: bool = None,
    ):
        """Gradient-descent tomography; see the module docstring for what runs
        where and which options raise."""
        self.set_device(device, clear_fft_cache)
        self._require_gpu()
        (use_projection, pa, pb, pc, parameter, step_size) = method_parameters(
            reconstruction_method, reconstruction_parameter, reconstruction_parameter_a,
            reconstruction_parameter_b, reconstruction_parameter_c, step_size)
        self._unsupported(
            projection_sets=use_projection, position_correction=not fix_positions,
            butterworth_filter=butterworth_filter and (q_lowpass is not None
                                                        or q_highpass is not None),
            tv_denoise=tv_denoise and tv_denoise_weights is not None,
            fit_probe_aberrations=fit_probe_aberrations and not fix_probe,
            constrain_probe_fourier_amplitude=constrain_probe_fourier_amplitude and not fix_probe,
            global_affine_transformation=global_affine_transformation and not fix_positions)
        self._reset_tomography(store_iterations, reset)
        self._report(num_iter, use_projection, reconstruction_method, parameter, pa, pb, pc,
                     normalization_min, max_batch_size, step_size)

        torch = engine._torch()
        n_meas = self._num_measurements
        cum = self._cum_probes_per_measurement
        if max_batch_size is not None:
            np.random.seed(seed_random)
        else:
            max_batch_size = int(self._num_diffraction_patterns)
        amplitudes = self._amplitudes_for_state()
        if amplitudes is None:
            raise ValueError("no diffraction amplitudes: call preprocess() with a datacube first")
        dev = torch.device("cuda", torch.cuda.current_device())
        if isinstance(amplitudes, torch.Tensor):
            amps_dev = amplitudes.to(device=dev, dtype=torch.float32).contiguous()
        else:
            amps_dev = torch.from_numpy(np.ascontiguousarray(amplitudes, dtype=np.float32)).to(dev)

        T = self._num_slices
        # a batch never spans tilts: the workspace holds the largest batch one tilt
        # forms (max_batch_size=None means the whole scan, i.e. each tilt in one batch)
        largest_tilt = int(np.max(np.diff(cum))) if n_meas else 1
        ws_batch = max(1, min(int(max_batch_size), largest_tilt))
        vol = torch.from_numpy(np.ascontiguousarray(self._object, dtype=np.float32)).to(dev)
        ops = VolumeOps(vol.shape, T, dev)
        roi = tuple(int(v) for v in self._region_of_interest_shape)
        sliced_np = np.zeros((T,) + tuple(vol.shape[1:]), dtype=np.float32)
        states, drivers = [], []
        for index in range(n_meas):
            start, end = int(cum[index]), int(cum[index + 1])
            if index == 0:
                st = engine.create_state(
                    roi_shape=roi, object_array=sliced_np, probe_array=self._probes_all[0],
                    amplitudes=amps_dev[start:end], positions_px=self._positions_px_all[start:end],
                    num_slices=T, num_probes=1, potential=True, max_batch=ws_batch,
                    storage="gpu", propagators=self._propagator_arrays,
                    detector_mask=detector_fourier_mask)
                base = st
            else:
                # the slices, workspace, propagators and mask are shared by the tilts
                st = dataclasses.replace(
                    base,
                    probe=torch.from_numpy(np.ascontiguousarray(
                        self._probes_all[index], dtype=np.complex64).reshape((1,) + roi)).to(dev),
                    amplitudes=amps_dev[start:end],
                    positions=torch.from_numpy(np.ascontiguousarray(
                        self._positions_px_all[start:end], dtype=np.float32)).to(dev),
                    order=torch.arange(end - start, dtype=torch.int32, device=dev),
                    error_accum=torch.zeros(1, dtype=torch.float32, device=dev),
                    order_pinned=None, order_events=None, extra={})
            states.append(st)
            drivers.append(engine.IterationDriver(
                st, max_batch=ws_batch, step_size=step_size,
                normalization_min=normalization_min, fix_probe=fix_probe, positivity=False,
                fix_probe_com=False, object_constraints=False,
                mean_intensity=self._mean_diffraction_intensity[index], graph=False))
        sliced = base.object
        sliced_old = torch.empty_like(sliced)
        blur_px = (gaussian_filter_sigma / self.sampling[0]
                   if gaussian_filter and gaussian_filter_sigma is not None else None)

        def volume_constraints():
            # gaussian, then shrinkage and positivity (the 3D object constraints)
            if blur_px is not None:
                ops.gaussian(vol, blur_px, roi)
            ops.constraints(vol, shrinkage_rad, object_positivity)
        collective = torch.empty_like(vol) if collective_measurement_updates else None
        self._device_states = states

        error = 0.0
        for _ in range(num_iter):
            error = 0.0
            if collective is not None:
                collective.zero_()
            indices = np.arange(n_meas)
            np.random.shuffle(indices)
            old = np.eye(3)
            for index in indices:
                rot = self._tilt_orientation_matrices[index]
                ops.rotate(vol, vol, rot @ old.T, 0)
                ops.project(vol, sliced)
                sliced_old.copy_(sliced)
                start, end = int(cum[index]), int(cum[index + 1])
                shuffled = np.arange(start, end)
                np.random.shuffle(shuffled)
                drivers[index].iterate((shuffled - start).astype(np.int64))
                if collective is not None:
                    ops.expand(sliced, sliced_old, ops.update, 1)
                    ops.rotate(ops.update, collective, np.asarray(rot).T, 2)
                else:
                    ops.expand(sliced, sliced_old, vol, 2)
                    volume_constraints()
                old = rot
            ops.rotate(vol, vol, np.asarray(old).T, 0)
            if collective is not None:
                ops.add_scaled(vol, collective, n_meas)
                volume_constraints()
            # every tilt keeps its own error sum: one read-back per iteration.
            # float64 error as the reference forms it: float32 mean intensity
            # times the tilt's pattern count (an int64) is a float64
            sums = torch.cat([states[i].error_accum for i in indices]).cpu().numpy()
            for index, batch_sum in zip(indices, sums):
                count = np.float64(cum[index + 1] - cum[index])
                error += float(batch_sum) / (
                    np.float64(self._mean_diffraction_intensity[index]) * count)
            error /= n_meas
            self.error_iterations.append(float(error))
            if store_iterations:
                self.object_iterations.append(vol.cpu().numpy())
                self.probe_iterations.append(
                    [np.fft.fftshift(s.probe.cpu().numpy()[0], axes=(-2, -1)) for s in states])

        self._object = vol.cpu().numpy()
        self._probes_all = [s.probe.cpu().numpy().reshape(roi) for s in states]
        self.object = self._object.copy()
        self.probe = self.probe_centered
        self.error = float(error)
        self._exit_waves = None
        self._volume_launches = ops.launches
        return self
