"""Drop-in reconstruction classes: SingleslicePtychography, MultislicePtychography and
MixedstatePtychography with the constructor, preprocess() and reconstruct()
signatures of py4DSTEM 0.14.18 (singleslice_ptychography.py:118-996,
multislice_ptychography.py:140-1115, mixedstate_ptychography.py:119-1027).

reconstruct() runs on the GPU through libptycho_gb300; there is no CPU path.
``device`` therefore accepts only "gpu" (the default here); "cpu" raises
ValueError. ``storage`` selects where the diffraction amplitudes live between
batches: "gpu" (resident in HBM) or "cpu" (host memory, one copy per batch as in
the reference's storage="cpu" mode).

Plotting arguments are accepted and ignored (this package draws nothing).
Options whose kernels are not implemented raise NotImplementedError rather than
silently changing the result.
"""

from __future__ import annotations

import warnings
from typing import Mapping, Sequence, Tuple, Union

import numpy as np

from . import engine
from .optics import POLAR_ALIASES, POLAR_SYMBOLS, ComplexProbe, electron_wavelength_angstrom
from .optics import resolve_polar_parameters, spatial_frequencies
from .preprocess import PreprocessMixin

warnings.simplefilter("always", UserWarning)


def method_parameters(reconstruction_method, reconstruction_parameter, a, b, c, step_size):
    """Map a method name to (use_projection, a, b, c, parameter, step)
    (phase_base_class.py:2005-2108)."""
    m = reconstruction_method
    if m == "generalized-projections":
        if a is None or b is None or c is None:
            raise ValueError(
                "reconstruction_parameter_a/b/c must all be specified "
                "when using reconstruction_method='generalized-projections'.")
        return True, a, b, c, None, None
    if m in ("DM_AP", "difference-map_alternating-projections"):
        if reconstruction_parameter < 0.0 or reconstruction_parameter > 1.0:
            raise ValueError("reconstruction_parameter must be between 0-1.")
        return True, -reconstruction_parameter, 1, 1 + reconstruction_parameter, \
            reconstruction_parameter, None
    if m in ("RAAR", "relaxed-averaged-alternating-reflections"):
        if reconstruction_parameter < 0.0 or reconstruction_parameter > 1.0:
            raise ValueError("reconstruction_parameter must be between 0-1.")
        return True, 1 - 2 * reconstruction_parameter, reconstruction_parameter, 2, \
            reconstruction_parameter, None
    if m in ("RRR", "relax-reflect-reflect"):
        if reconstruction_parameter < 0.0 or reconstruction_parameter > 2.0:
            raise ValueError("reconstruction_parameter must be between 0-2.")
        return True, -reconstruction_parameter, reconstruction_parameter, 2, \
            reconstruction_parameter, None
    if m in ("SUPERFLIP", "charge-flipping"):
        return True, 0, 1, 2, None, None
    if m in ("GD", "gradient-descent"):
        return False, None, None, None, None, step_size
    raise ValueError(
        "reconstruction_method must be one of 'generalized-projections', "
        "'DM_AP' (or 'difference-map_alternating-projections'), "
        "'RAAR' (or 'relaxed-averaged-alternating-reflections'), "
        "'RRR' (or 'relax-reflect-reflect'), "
        "'SUPERFLIP' (or 'charge-flipping'), "
        f"or 'GD' (or 'gradient-descent'), not  {reconstruction_method}.")


class _PtychographyBase(PreprocessMixin):
    """State and behaviour common to the three reconstruction classes."""

    _num_slices = 1
    _num_probes = 1
    _multislice = False
    _mixed = False

    # -- construction ----------------------------------------------------------
    def _common_init(self, energy, datacube, semiangle_cutoff, semiangle_cutoff_pixels,
                     rolloff, vacuum_probe_intensity, polar_parameters, initial_object_guess,
                     initial_probe_guess, initial_scan_positions, object_fov_ang,
                     positions_offset_ang, object_padding_px, object_type, positions_mask,
                     verbose, device, storage, clear_fft_cache, name, kwargs):
        self.name = name
        if storage is None:
            storage = device
        self.set_device(device, clear_fft_cache)
        self.set_storage(storage)
        for key in kwargs:
            if key not in POLAR_SYMBOLS and key not in POLAR_ALIASES:
                raise ValueError("{} not a recognized parameter".format(key))
        self._polar_parameters = dict(zip(POLAR_SYMBOLS, [0.0] * len(POLAR_SYMBOLS)))
        params = {} if polar_parameters is None else polar_parameters
        params.update(kwargs)
        resolve_polar_parameters(params, self._polar_parameters)
        if object_type != "potential" and object_type != "complex":
            raise ValueError(
                f"object_type must be either 'potential' or 'complex', not {object_type}")
        self.set_save_defaults()
        self._datacube = datacube
        self._object = initial_object_guess
        self._probe = initial_probe_guess
        self._vacuum_probe_intensity = vacuum_probe_intensity
        self._scan_positions = initial_scan_positions
        self._positions_offset_ang = positions_offset_ang
        self._energy = energy
        self._semiangle_cutoff = semiangle_cutoff
        self._semiangle_cutoff_pixels = semiangle_cutoff_pixels
        self._rolloff = rolloff
        self._object_type = object_type
        self._object_padding_px = object_padding_px
        self._object_fov_ang = object_fov_ang
        self._positions_mask = positions_mask
        self._verbose = verbose
        self._preprocessed = False
        self._exit_waves = None
        # replay each iteration from one captured CUDA graph (eager issue when False)
        self._graph_iterations = True

    def set_device(self, device, clear_fft_cache):
        if clear_fft_cache is not None:
            self._clear_fft_cache = clear_fft_cache
        if device is None:
            return self
        if device not in ("cpu", "gpu"):
            raise ValueError(f"device must be either 'cpu' or 'gpu', not {device}")
        self._device = device
        return self

    def _require_gpu(self):
        """device="cpu" runs preprocess() on the host (NumPy); everything after it
        runs on the GPU only."""
        if self._device != "gpu":
            raise ValueError(
                "py4dstem_gb300 reconstructs on the GPU only: pass device='gpu' "
                "(device='cpu' runs preprocess() on the host; the CPU reconstruction is "
                "the reference implementation)")

    # Amplitudes preprocessed on the device stay there; the host copy is made
    # the first time something asks for it.
    @property
    def _amplitudes(self):
        host = self.__dict__.get("_amplitudes_host")
        if host is None and self.__dict__.get("_amplitudes_device") is not None:
            host = self._amplitudes_device.cpu().numpy()
            self.__dict__["_amplitudes_host"] = host
        return host

    @_amplitudes.setter
    def _amplitudes(self, value):
        self.__dict__["_amplitudes_host"] = value
        self.__dict__["_amplitudes_device"] = None

    def _set_device_amplitudes(self, amps):
        if self._storage == "cpu":
            # host storage: one copy into page-locked memory, from which each
            # batch's patterns are gathered to the device one batch ahead; the
            # device copy is released
            import torch

            host = torch.empty(tuple(amps.shape), dtype=amps.dtype, pin_memory=True)
            host.copy_(amps)
            self.__dict__["_amplitudes_host"] = host.numpy()
            self.__dict__["_amplitudes_device"] = None
            return
        self.__dict__["_amplitudes_host"] = None
        self.__dict__["_amplitudes_device"] = amps

    def _amplitudes_for_state(self):
        """The amplitudes as create_state takes them: the device tensor when the
        preprocessing left one and storage is "gpu", else the host array. With
        storage "cpu" a pageable host array is moved once into page-locked memory
        (kept for later calls), so that each batch's patterns are gathered to the
        device over the CPU-GPU link, one batch ahead on a second stream, instead
        of staging every batch through a host-side gather and copy."""
        dev = self.__dict__.get("_amplitudes_device")
        if dev is not None and self._storage == "gpu":
            return dev
        host = self._amplitudes
        if self._storage == "cpu" and self._device == "gpu" and host is not None \
                and engine.mapped_host_address(np.ascontiguousarray(host)) is None:
            import torch

            pinned = torch.empty(tuple(host.shape), dtype=torch.float32, pin_memory=True)
            pinned.numpy()[...] = host
            host = pinned.numpy()
            self.__dict__["_amplitudes_host"] = host
        return host

    def set_storage(self, storage):
        if storage not in ("cpu", "gpu"):
            raise ValueError(f"storage must be either 'cpu' or 'gpu', not {storage}")
        self._storage = storage
        return self

    def save(self, path):
        """Write this reconstruction to `path` (.npz; see py4dstem_gb300.io)."""
        from . import io

        io.save(path, self)

    def set_save_defaults(self, save_datacube=False, save_exit_waves=False,
                          save_iterations=True, save_iterations_frequency=1):
        self._save_datacube = save_datacube
        self._save_exit_waves = save_exit_waves
        self._save_iterations = save_iterations
        self._save_iterations_frequency = save_iterations_frequency
        return self

    def attach_datacube(self, datacube):
        self._datacube = datacube
        return self

    def reinitialize_parameters(self, device=None, storage=None, clear_fft_cache=None,
                                verbose=None):
        if device is not None:
            self.set_device(device, clear_fft_cache)
        if storage is not None:
            self.set_storage(storage)
        if verbose is not None:
            self._verbose = verbose
        return self

    # -- properties ------------------------------------------------------------
    @property
    def angular_sampling(self):
        return getattr(self, "_angular_sampling", None)

    @property
    def sampling(self):
        if self.angular_sampling is None:
            return None
        lam = electron_wavelength_angstrom(self._energy)
        return tuple(lam * 1e3 / dk / n for dk, n in zip(self.angular_sampling,
                                                         self._amplitudes_shape))

    @property
    def positions(self):
        if self.angular_sampling is None:
            return None
        pos = np.array(self._positions_px, copy=True)
        pos[:, 0] *= self.sampling[0]
        pos[:, 1] *= self.sampling[1]
        return pos

    @property
    def probe_centered(self):
        if getattr(self, "_probe", None) is None:
            return None
        return np.fft.fftshift(np.asarray(self._probe, dtype=np.complex64), axes=(-2, -1))

    @property
    def probe_fourier(self):
        if getattr(self, "_probe", None) is None:
            return None
        return np.fft.fftshift(np.fft.fft2(np.asarray(self._probe, dtype=np.complex64)),
                               axes=(-2, -1))

    def _single_probe_array(self):
        p = np.asarray(self._probe)
        return p[0] if self._mixed else p

    # -- preprocess ------------------------------------------------------------
    def _preprocess_impl(self, diffraction_intensities_shape, reshaping_method,
                         padded_diffraction_intensities_shape, region_of_interest_shape,
                         dp_mask, in_place_datacube_modification, fit_function,
                         maximize_divergence, rotation_angles_deg, force_com_rotation,
                         force_com_transpose, force_com_shifts, force_com_measured,
                         vectorized_com_calculation, force_scan_sampling,
                         force_angular_sampling, force_reciprocal_sampling, object_fov_mask,
                         crop_patterns, center_positions_in_fov, store_initial_arrays, device,
                         clear_fft_cache, max_batch_size):
        self.set_device(device, clear_fft_cache)
        self._diffraction_intensities_shape = diffraction_intensities_shape
        self._reshaping_method = reshaping_method
        self._padded_diffraction_intensities_shape = padded_diffraction_intensities_shape
        self._dp_mask = dp_mask
        if self._datacube is None:
            raise ValueError(
                "The preprocess() method requires a DataCube. "
                "Please run ptycho.attach_datacube(DataCube) first.")
        if self._positions_mask is not None:
            self._positions_mask = np.asarray(self._positions_mask, dtype="bool")

        (self._datacube, self._vacuum_probe_intensity, self._dp_mask, force_com_shifts,
         force_com_measured) = self._prepare_datacube(
            self._datacube, diffraction_intensities_shape, reshaping_method,
            padded_diffraction_intensities_shape, self._vacuum_probe_intensity, self._dp_mask,
            force_com_shifts, force_com_measured)

        intensities = self._intensities_and_calibrations(
            self._datacube, force_scan_sampling, force_angular_sampling,
            force_reciprocal_sampling)
        if self._semiangle_cutoff_pixels:
            self._semiangle_cutoff = self._semiangle_cutoff_pixels * self._angular_sampling[0]

        # device="gpu": the per-pattern steps run on the device copy of the patterns
        intensities_dev = None
        if self._device == "gpu":
            from . import device_preprocess

            intensities_dev = device_preprocess.upload_intensities(intensities)

        (self._com_measured_x, self._com_measured_y, self._com_fitted_x, self._com_fitted_y,
         self._com_normalized_x, self._com_normalized_y) = self._intensities_center_of_mass(
            intensities, self._dp_mask, fit_function, force_com_shifts, force_com_measured,
            vectorized_com_calculation, intensities_dev)

        (self._rotation_best_rad, self._rotation_best_transpose, self._com_x,
         self._com_y) = self._solve_rotation(
            self._com_normalized_x, self._com_normalized_y, rotation_angles_deg,
            maximize_divergence, force_com_rotation, force_com_transpose)

        if intensities_dev is not None:
            (amps, self._mean_diffraction_intensity, self._crop_mask,
             self._crop_mask_shape) = self._normalize_intensities_device(
                intensities_dev, self._com_fitted_x, self._com_fitted_y, self._positions_mask,
                crop_patterns)
            del intensities_dev
            self._set_device_amplitudes(amps)
        else:
            (self._amplitudes, self._mean_diffraction_intensity, self._crop_mask,
             self._crop_mask_shape) = self._normalize_intensities(
                intensities, self._com_fitted_x, self._com_fitted_y, self._positions_mask,
                crop_patterns, in_place_datacube_modification)
        del intensities

        amp_shape = tuple(self._amplitudes_for_state().shape)
        self._num_diffraction_patterns = amp_shape[0]
        self._amplitudes_shape = np.array(amp_shape[-2:])
        # region_of_interest_shape (singleslice_ptychography.py:431-436): the probe
        # and the object patches take that shape and every Fourier projection
        # resamples the far field between it and the detector grid
        if region_of_interest_shape is not None:
            self._resample_exit_waves = True
            self._region_of_interest_shape = np.array(region_of_interest_shape)
        else:
            self._resample_exit_waves = False
            self._region_of_interest_shape = np.array(amp_shape[-2:])

        self._positions_px, self._object_padding_px = self._scan_positions_in_pixels(
            self._scan_positions, self._positions_mask, self._object_padding_px,
            self._positions_offset_ang)

        self._object = self._initial_object(
            self._object, self._positions_px, self._object_type,
            self._num_slices if self._multislice else None)
        if store_initial_arrays:
            self._object_initial = self._object.copy()
            self._object_type_initial = self._object_type
        self._object_shape = self._object.shape[-2:] if self._multislice else self._object.shape

        self._positions_px = np.asarray(self._positions_px, dtype=np.float32)
        self._positions_px_initial_com = self._positions_px.mean(0)
        if center_positions_in_fov:
            self._positions_px -= (self._positions_px_initial_com
                                   - np.array(self._object_shape) / 2)
            self._positions_px_initial_com = self._positions_px.mean(0)
        self._positions_px_initial = self._positions_px.copy()
        self._positions_initial = self._positions_px_initial.copy()
        self._positions_initial[:, 0] *= self.sampling[0]
        self._positions_initial[:, 1] *= self.sampling[1]

        init_probe = self._mixed_probes if self._mixed else self._single_probe
        self._probe, self._semiangle_cutoff = init_probe(
            self._probe, self._vacuum_probe_intensity, self._mean_diffraction_intensity,
            self._semiangle_cutoff, crop_patterns)

        self._known_aberrations_array = ComplexProbe(
            energy=self._energy, gpts=self._region_of_interest_shape, sampling=self.sampling,
            parameters=self._polar_parameters).evaluate_ctf()
        if store_initial_arrays:
            self._probe_initial = self._probe.copy()
            self._probe_initial_aperture = np.abs(np.fft.fft2(self._probe))
        else:
            self._probe_initial_aperture = None

        if self._multislice:
            self._propagator_arrays = self._fresnel_propagators()

        if object_fov_mask is None:
            overlap = self._probe_overlap(self._single_probe_array(), max_batch_size)
        else:
            overlap = None
        self._object_fov_mask = self._fov_mask(object_fov_mask, overlap)
        self._object_fov_mask_inverse = np.invert(self._object_fov_mask)
        self._preprocessed = True
        return self

    # -- reconstruct -----------------------------------------------------------
    def _reset_reconstruction(self, store_iterations, reset):
        if store_iterations and (not hasattr(self, "object_iterations") or reset):
            self.object_iterations = []
            self.probe_iterations = []
        if reset is True:
            self.error_iterations = []
            self._object = self._object_initial.copy()
            self._probe = self._probe_initial.copy()
            self._positions_px = self._positions_px_initial.copy()
            self._object_type = self._object_type_initial
            self._exit_waves = None
        elif reset is None:
            if hasattr(self, "error"):
                warnings.warn("Continuing reconstruction from previous result. "
                              "Use reset=True for a fresh start.", UserWarning)
            else:
                self.error_iterations = []
                self._exit_waves = None
        else:
            if not hasattr(self, "error"):
                self.error_iterations = []
                self._exit_waves = None

    def _switch_object_type(self, object_type):
        if (self._object_type, object_type) == ("potential", "complex"):
            self._object_type = "complex"
            self._object = np.exp(1j * self._object, dtype=np.complex64)
        elif (self._object_type, object_type) == ("complex", "potential"):
            self._object_type = "potential"
            self._object = np.angle(self._object)
        return self

    def _report(self, num_iter, use_projection, method, parameter, a, b, c, normalization_min,
                max_batch_size, step_size):
        first = (f"Performing {num_iter} iterations using a {self._object_type} object type, ")
        if max_batch_size is not None:
            if use_projection:
                raise ValueError(
                    "Stochastic object/probe updating is inconsistent with 'DM_AP', 'RAAR', "
                    "'RRR', and 'SUPERFLIP'. Use reconstruction_method='GD' or set "
                    "max_batch_size=None.")
            msg = (first + f"with the {method} algorithm, with normalization_min: "
                   f"{normalization_min} and step _size: {step_size}, in batches of max "
                   f"{max_batch_size} measurements.")
        elif parameter is not None:
            msg = (first + f"with the {method} algorithm, with normalization_min: "
                   f"{normalization_min} and α: {parameter}.")
        elif a is not None:
            msg = (first + f"with the {method} algorithm, with normalization_min: "
                   f"{normalization_min} and (a,b,c): {a, b, c}.")
        else:
            msg = (first + f"with the {method} algorithm, with normalization_min: "
                   f"{normalization_min} and step _size: {step_size}.")
        if self._verbose:
            warnings.warn(msg, UserWarning)

    @staticmethod
    def _unsupported(**flags):
        for name, on in flags.items():
            if on:
                raise NotImplementedError(
                    f"reconstruct option {name!r} has no GPU implementation in py4dstem_gb300")

    def _reconstruct_impl(self, *, num_iter, reconstruction_method, reconstruction_parameter,
                          reconstruction_parameter_a, reconstruction_parameter_b,
                          reconstruction_parameter_c, max_batch_size, seed_random, step_size,
                          normalization_min, fix_probe_com, fix_probe, fix_positions,
                          fix_positions_com, positions_step_size, max_position_update_distance,
                          max_position_total_distance, pure_phase_object, object_positivity, shrinkage_rad,
                          fix_potential_baseline, detector_fourier_mask, store_iterations,
                          reset, device, clear_fft_cache, object_type,
                          orthogonalize_probe=False, fix_probe_aperture=False,
                          constrain_probe_amplitude=False,
                          constrain_probe_amplitude_relative_radius=0.5,
                          constrain_probe_amplitude_relative_width=0.05,
                          identical_slices=False, gaussian_filter_sigma=None,
                          global_affine_transformation=False, unsupported=None):
        self.set_device(device, clear_fft_cache)
        self._require_gpu()
        self._reset_reconstruction(store_iterations, reset)
        if object_type is not None:
            self._switch_object_type(object_type)
        (use_projection, pa, pb, pc, parameter, step_size) = method_parameters(
            reconstruction_method, reconstruction_parameter, reconstruction_parameter_a,
            reconstruction_parameter_b, reconstruction_parameter_c, step_size)
        self._report(num_iter, use_projection, reconstruction_method, parameter, pa, pb, pc,
                     normalization_min, max_batch_size, step_size)
        self._unsupported(**(unsupported or {}))
        if use_projection and detector_fourier_mask is not None:
            raise NotImplementedError()
        correct_positions = not fix_positions

        J = self._num_diffraction_patterns
        shuffled = np.arange(J)
        if max_batch_size is not None:
            np.random.seed(seed_random)
        else:
            max_batch_size = J

        potential = self._object_type == "potential"
        obj = np.asarray(self._object, dtype=np.float32 if potential else np.complex64)
        # (the reference's mask.sum() > 0, as a test for any set pixel)
        use_mask = bool(fix_potential_baseline and self._object_fov_mask_inverse.any())
        amplitudes = self._amplitudes_for_state()
        if amplitudes is None:
            raise ValueError("no diffraction amplitudes: call preprocess() with a datacube first "
                             "(an object from py4dstem_gb300.read() keeps no amplitudes)")
        driver_kw = dict(
            max_batch=int(max_batch_size), projection=use_projection, step_size=step_size,
            normalization_min=normalization_min, fix_probe=fix_probe,
            projection_abc=(pa, pb, pc), shrinkage_rad=shrinkage_rad, use_mask=use_mask,
            pure_phase=pure_phase_object and self._object_type == "complex",
            positivity=object_positivity, fix_probe_com=fix_probe_com,
            orthogonalize_probe=orthogonalize_probe,
            mean_intensity=self._mean_diffraction_intensity, graph=self._graph_iterations,
            position_correction=(dict(
                step_size=positions_step_size,
                max_update_px=self._distance_px(max_position_update_distance),
                max_total_px=self._distance_px(max_position_total_distance),
                # the reference passes fix_positions_com and not fix_positions on
                # (singleslice_ptychography.py:956, ptychographic_constraints.py:1355-1377)
                center_of_mass=not fix_positions_com,
                affine=global_affine_transformation) if correct_positions else None))
        # optional constraints: the initial probe's Fourier amplitude (mode 0) and the
        # soft top-hat of the amplitude constraint (ptychographic_constraints.py:920-957)
        aperture = amp_mask = None
        if fix_probe_aperture:
            if self._probe_initial_aperture is None:
                raise ValueError("fix_probe_aperture needs preprocess(store_initial_arrays=True)")
            aperture = np.asarray(self._probe_initial_aperture)
            aperture = aperture[0] if aperture.ndim == 3 else aperture
        if constrain_probe_amplitude:
            from scipy.special import erf

            sx, sy = (int(v) for v in self._region_of_interest_shape)
            X = np.fft.fftfreq(sx)[:, None]
            Y = np.fft.fftfreq(sy)[None]
            r = np.hypot(X, Y) - constrain_probe_amplitude_relative_radius
            sigma = np.sqrt(np.pi) / constrain_probe_amplitude_relative_width
            amp_mask = 0.5 * (1 - erf(sigma * r / (1 - r ** 2)))
        gaussian = None
        pure_phase = pure_phase_object and self._object_type == "complex"
        if gaussian_filter_sigma is not None:
            # scipy.ndimage.gaussian_filter's kernel (truncate 4) for the sigma in
            # pixels (ptychographic_constraints.py:141)
            sigma = gaussian_filter_sigma / self.sampling[0]
            if sigma > 1e-15:
                radius = int(4.0 * sigma + 0.5)
                x = np.arange(-radius, radius + 1)
                phi = np.exp(-0.5 / (sigma * sigma) * x ** 2)
                gaussian = (phi / phi.sum(), pure_phase)
        constraint_key = (None if gaussian is None else (gaussian_filter_sigma, pure_phase),
                          fix_probe_aperture, id(self._probe_initial_aperture),
                          constrain_probe_amplitude, constrain_probe_amplitude_relative_radius,
                          constrain_probe_amplitude_relative_width, bool(identical_slices))
        # Device state and iteration driver are kept between calls with the same
        # arrays and settings: a later call copies the current object, probe and
        # positions into the same buffers and replays the iteration graph captured
        # before (the reference rebuilds nothing on the device either).
        key = (self._storage, obj.shape, obj.dtype.str, np.shape(self._probe),
               self._num_slices, self._num_probes, potential, self._mixed, correct_positions,
               detector_fourier_mask is not None, constraint_key,
               repr(sorted((k, repr(v)) for k, v in driver_kw.items())))
        cached = self.__dict__.get("_state_cache")
        refresh = cached is not None and cached[0] == key and cached[1] is amplitudes
        if refresh:
            st, driver = cached[2], cached[3]
        else:
            self.__dict__["_state_cache"] = None  # release the previous buffers first
            st = engine.create_state(
                roi_shape=tuple(self._region_of_interest_shape), object_array=obj,
                probe_array=self._probe, amplitudes=amplitudes,
                positions_px=self._positions_px, num_slices=self._num_slices,
                num_probes=self._num_probes, potential=potential,
                max_batch=int(max_batch_size), storage=self._storage,
                propagators=(getattr(self, "_propagator_arrays", None)
                             if self._multislice else None),
                detector_mask=detector_fourier_mask,
                fov_mask_inverse=self._object_fov_mask_inverse if use_mask else None,
                projection=use_projection, mixed_state=self._mixed,
                positions_initial=self._positions_px_initial if correct_positions else None)
            driver = engine.IterationDriver(st, identical_slices=identical_slices,
                                            probe_aperture=aperture,
                                            probe_amplitude_mask=amp_mask, gaussian=gaussian,
                                            **driver_kw)
            self.__dict__["_state_cache"] = (key, amplitudes, st, driver)
        if num_iter > 0 and not use_projection:
            np.random.shuffle(shuffled)
        if num_iter > 0:
            # with host-resident amplitudes the first batch's patterns start
            # crossing the CPU-GPU link now, while the host copies the arrays in
            driver.prefetch(shuffled)
        if refresh:
            engine.refresh_state(
                st, object_array=obj, probe_array=self._probe, positions_px=self._positions_px,
                detector_mask=detector_fourier_mask,
                fov_mask_inverse=self._object_fov_mask_inverse if use_mask else None,
                positions_initial=self._positions_px_initial if correct_positions else None)
        if use_projection:
            if self._exit_waves is not None:
                import torch

                st.exit_waves.copy_(torch.from_numpy(np.asarray(
                    self._exit_waves, dtype=np.complex64).reshape(st.exit_waves.shape)))
                st.exit_waves_valid = True
            else:
                st.exit_waves_valid = False
        self._device_state = st
        error = np.float32(0.0)
        for it in range(num_iter):
            driver.iterate(shuffled)
            # the next iteration's shuffle (same global-RNG sequence as the
            # reference) runs on the host while the GPU works on this one
            if it + 1 < num_iter and not use_projection:
                np.random.shuffle(shuffled)
            error = driver.error()
            self.error_iterations.append(error.item())
            if store_iterations:
                self.object_iterations.append(st.object.cpu().numpy().copy())
                self.probe_iterations.append(
                    np.fft.fftshift(st.probe.cpu().numpy().reshape(np.shape(self._probe)),
                                    axes=(-2, -1)))

        self._object = st.object.cpu().numpy()
        self.object = st.object.cpu().numpy()  # a second transfer, not a host copy
        self._probe = st.probe.cpu().numpy().reshape(np.shape(self._probe))
        if correct_positions:
            self._positions_px = st.positions.cpu().numpy()
            if driver.affine is not None:
                self._tf = driver.affine
        self.probe = self.probe_centered
        self.error = error.item()
        if use_projection:
            self._exit_waves = st.exit_waves.cpu().numpy()
        else:
            self._exit_waves = None
        return self

    def _distance_px(self, distance_ang):
        """A distance limit in A as pixels, like the reference's
        distance / sqrt(sx^2 + sy^2) (ptychographic_methods.py:2191-2213); None stays None."""
        if distance_ang is None:
            return None
        return float(distance_ang / np.sqrt(self.sampling[0] ** 2 + self.sampling[1] ** 2))

    def _return_self_consistency_errors(self, max_batch_size=None):
        """Per-position self-consistency errors of the current object and probe
        (ptychographic_methods.py:2227-2291): sum (A - |F|)^2 of a forward-only GPU
        pass in natural position order, divided by the mean intensity (float64)."""
        self._require_gpu()
        potential = self._object_type == "potential"
        J = self._num_diffraction_patterns
        max_batch_size = J if max_batch_size is None else int(max_batch_size)
        st = engine.create_state(
            roi_shape=tuple(self._region_of_interest_shape),
            object_array=np.asarray(self._object, dtype=np.float32 if potential else np.complex64),
            probe_array=self._probe, amplitudes=self._amplitudes_for_state(),
            positions_px=self._positions_px, num_slices=self._num_slices,
            num_probes=self._num_probes, potential=potential, max_batch=max_batch_size,
            storage=self._storage,
            propagators=getattr(self, "_propagator_arrays", None) if self._multislice else None,
            mixed_state=self._mixed)
        errors = engine.self_consistency_errors(st, max_batch_size)
        return errors.astype(np.float64) / self._mean_diffraction_intensity

    def _fresnel_propagators(self):
        """(T-1, Sx, Sy) complex64 Fresnel propagators with optional tilt
        (ptychographic_methods.py:318-381)."""
        kx, ky = spatial_frequencies(self._region_of_interest_shape, self.sampling)
        lam = electron_wavelength_angstrom(self._energy)
        thick = self._slice_thicknesses
        props = np.empty((thick.shape[0], kx.shape[0], ky.shape[0]), dtype=np.complex64)
        for i, dz in enumerate(thick):
            props[i] = np.exp(1.0j * (-(kx**2)[:, None] * np.pi * lam * dz))
            props[i] *= np.exp(1.0j * (-(ky**2)[None] * np.pi * lam * dz))
            if self._theta_x is not None:
                props[i] *= np.exp(1.0j * (-2 * kx[:, None] * np.pi * dz * np.tan(self._theta_x / 1e3)))
            if self._theta_y is not None:
                props[i] *= np.exp(1.0j * (-2 * ky[None] * np.pi * dz * np.tan(self._theta_y / 1e3)))
        return props


_PREPROCESS_DOC = """Preprocess the datacube: calibrations, centre of mass and rotation,
corner-centred amplitudes, scan positions and the initial object, probe and
FOV mask. Same arguments as the reference's preprocess(); plot_* are ignored."""


class SingleslicePtychography(_PtychographyBase):
    """Single-slice ptychography (object (Px,Py), probe (Sx,Sy))."""

    def __init__(
        self,
        energy: float,
        datacube=None,
        semiangle_cutoff: float = None,
        semiangle_cutoff_pixels: float = None,
        rolloff: float = 2.0,
        vacuum_probe_intensity: np.ndarray = None,
        polar_parameters: Mapping[str, float] = None,
        initial_object_guess: np.ndarray = None,
        initial_probe_guess: np.ndarray = None,
        initial_scan_positions: np.ndarray = None,
        object_fov_ang: Tuple[float, float] = None,
        positions_offset_ang: np.ndarray = None,
        object_padding_px: Tuple[int, int] = None,
        object_type: str = "complex",
        positions_mask: np.ndarray = None,
        verbose: bool = True,
        device: str = "gpu",
        storage: str = None,
        clear_fft_cache: bool = True,
        name: str = "ptychographic_reconstruction",
        **kwargs,
    ):
        self._common_init(energy, datacube, semiangle_cutoff, semiangle_cutoff_pixels, rolloff,
                          vacuum_probe_intensity, polar_parameters, initial_object_guess,
                          initial_probe_guess, initial_scan_positions, object_fov_ang,
                          positions_offset_ang, object_padding_px, object_type, positions_mask,
                          verbose, device, storage, clear_fft_cache, name, kwargs)

    def preprocess(
        self,
        diffraction_intensities_shape: Tuple[int, int] = None,
        reshaping_method: str = "bilinear",
        padded_diffraction_intensities_shape: Tuple[int, int] = None,
        region_of_interest_shape: Tuple[int, int] = None,
        dp_mask: np.ndarray = None,
        in_place_datacube_modification: bool = False,
        fit_function: str = "plane",
        plot_center_of_mass: str = "default",
        plot_rotation: bool = True,
        maximize_divergence: bool = False,
        rotation_angles_deg: np.ndarray = None,
        plot_probe_overlaps: bool = True,
        force_com_rotation: float = None,
        force_com_transpose: float = None,
        force_com_shifts: Union[Sequence[np.ndarray], Sequence[float]] = None,
        force_com_measured: Sequence[np.ndarray] = None,
        vectorized_com_calculation: bool = True,
        force_scan_sampling: float = None,
        force_angular_sampling: float = None,
        force_reciprocal_sampling: float = None,
        object_fov_mask: np.ndarray = None,
        crop_patterns: bool = False,
        center_positions_in_fov: bool = True,
        store_initial_arrays: bool = True,
        device: str = None,
        clear_fft_cache: bool = None,
        max_batch_size: int = None,
        **kwargs,
    ):
        return self._preprocess_impl(
            diffraction_intensities_shape, reshaping_method, padded_diffraction_intensities_shape,
            region_of_interest_shape, dp_mask, in_place_datacube_modification, fit_function,
            maximize_divergence, rotation_angles_deg, force_com_rotation, force_com_transpose,
            force_com_shifts, force_com_measured, vectorized_com_calculation,
            force_scan_sampling, force_angular_sampling, force_reciprocal_sampling,
            object_fov_mask, crop_patterns, center_positions_in_fov, store_initial_arrays,
            device, clear_fft_cache, max_batch_size)

    preprocess.__doc__ = _PREPROCESS_DOC

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
        positions_step_size: float = 0.5,
        pure_phase_object: bool = False,
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
        tv_denoise: bool = True,
        tv_denoise_weight: float = None,
        tv_denoise_inner_iter: float = 40,
        object_positivity: bool = True,
        shrinkage_rad: float = 0.0,
        fix_potential_baseline: bool = True,
        detector_fourier_mask: np.ndarray = None,
        store_iterations: bool = False,
        progress_bar: bool = True,
        reset: bool = None,
        device: str = None,
        clear_fft_cache: bool = None,
        object_type: str = None,
    ):
        """Run `num_iter` iterations on the GPU; returns self with `object`,
        `probe` (centred), `error` and `error_iterations` set."""
        return self._reconstruct_impl(
            num_iter=num_iter, reconstruction_method=reconstruction_method,
            reconstruction_parameter=reconstruction_parameter,
            reconstruction_parameter_a=reconstruction_parameter_a,
            reconstruction_parameter_b=reconstruction_parameter_b,
            reconstruction_parameter_c=reconstruction_parameter_c,
            max_batch_size=max_batch_size, seed_random=seed_random, step_size=step_size,
            normalization_min=normalization_min, fix_probe_com=fix_probe_com,
            fix_probe=fix_probe, fix_positions=fix_positions,
            fix_positions_com=fix_positions_com, positions_step_size=positions_step_size,
            max_position_update_distance=max_position_update_distance,
            max_position_total_distance=max_position_total_distance,
            pure_phase_object=pure_phase_object, object_positivity=object_positivity,
            shrinkage_rad=shrinkage_rad, fix_potential_baseline=fix_potential_baseline,
            detector_fourier_mask=detector_fourier_mask, store_iterations=store_iterations,
            reset=reset, device=device, clear_fft_cache=clear_fft_cache,
            object_type=object_type,
            fix_probe_aperture=fix_probe_aperture and not fix_probe,
            constrain_probe_amplitude=constrain_probe_amplitude and not fix_probe,
            constrain_probe_amplitude_relative_radius=constrain_probe_amplitude_relative_radius,
            constrain_probe_amplitude_relative_width=constrain_probe_amplitude_relative_width,
            gaussian_filter_sigma=gaussian_filter_sigma if gaussian_filter else None,
            global_affine_transformation=global_affine_transformation and not fix_positions,
            unsupported=dict(
                constrain_probe_fourier_amplitude=constrain_probe_fourier_amplitude
                and not fix_probe,
                fit_probe_aberrations=fit_probe_aberrations and not fix_probe,
                butterworth_filter=butterworth_filter
                and (q_lowpass is not None or q_highpass is not None),
                tv_denoise=tv_denoise and tv_denoise_weight is not None,
            ))


class MixedstatePtychography(_PtychographyBase):
    """Mixed-state ptychography (probe (M,Sx,Sy) incoherent modes)."""

    _mixed = True

    def __init__(
        self,
        energy: float,
        datacube=None,
        num_probes: int = None,
        semiangle_cutoff: float = None,
        semiangle_cutoff_pixels: float = None,
        rolloff: float = 2.0,
        vacuum_probe_intensity: np.ndarray = None,
        polar_parameters: Mapping[str, float] = None,
        object_padding_px: Tuple[int, int] = None,
        initial_object_guess: np.ndarray = None,
        initial_probe_guess: np.ndarray = None,
        initial_scan_positions: np.ndarray = None,
        object_fov_ang: Tuple[float, float] = None,
        positions_offset_ang: np.ndarray = None,
        object_type: str = "complex",
        positions_mask: np.ndarray = None,
        verbose: bool = True,
        device: str = "gpu",
        storage: str = None,
        clear_fft_cache: bool = True,
        name: str = "mixed-state_ptychographic_reconstruction",
        **kwargs,
    ):
        if initial_probe_guess is None or isinstance(initial_probe_guess, ComplexProbe):
            if num_probes is None:
                raise ValueError(
                    "If initial_probe_guess is None, or a ComplexProbe object, "
                    "num_probes must be specified.")
        else:
            if len(initial_probe_guess.shape) != 3:
                raise ValueError("Specified initial_probe_guess must have dimensions (N,Sx,Sy).")
            num_probes = initial_probe_guess.shape[0]
        self._common_init(energy, datacube, semiangle_cutoff, semiangle_cutoff_pixels, rolloff,
                          vacuum_probe_intensity, polar_parameters, initial_object_guess,
                          initial_probe_guess, initial_scan_positions, object_fov_ang,
                          positions_offset_ang, object_padding_px, object_type, positions_mask,
                          verbose, device, storage, clear_fft_cache, name, kwargs)
        self._num_probes = num_probes

    preprocess = SingleslicePtychography.preprocess

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
        pure_phase_object: bool = False,
        fix_probe_com: bool = True,
        orthogonalize_probe: bool = True,
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
        global_affine_transformation: bool = False,
        max_position_update_distance: float = None,
        max_position_total_distance: float = None,
        gaussian_filter_sigma: float = None,
        gaussian_filter: bool = True,
        fit_probe_aberrations: bool = False,
        fit_probe_aberrations_max_angular_order: int = 4,
        fit_probe_aberrations_max_radial_order: int = 4,
        fit_probe_aberrations_remove_initial: bool = False,
        fit_probe_aberrations_using_scikit_image: bool = True,
        num_probes_fit_aberrations: int = np.inf,
        butterworth_filter: bool = True,
        q_lowpass: float = None,
        q_highpass: float = None,
        butterworth_order: float = 2,
        tv_denoise: bool = True,
        tv_denoise_weight: float = None,
        tv_denoise_inner_iter: float = 40,
        object_positivity: bool = True,
        shrinkage_rad: float = 0.0,
        fix_potential_baseline: bool = True,
        detector_fourier_mask: np.ndarray = None,
        store_iterations: bool = False,
        progress_bar: bool = True,
        reset: bool = None,
        device: str = None,
        clear_fft_cache: bool = None,
        object_type: str = None,
    ):
        """Run `num_iter` mixed-state iterations on the GPU."""
        return self._reconstruct_impl(
            num_iter=num_iter, reconstruction_method=reconstruction_method,
            reconstruction_parameter=reconstruction_parameter,
            reconstruction_parameter_a=reconstruction_parameter_a,
            reconstruction_parameter_b=reconstruction_parameter_b,
            reconstruction_parameter_c=reconstruction_parameter_c,
            max_batch_size=max_batch_size, seed_random=seed_random, step_size=step_size,
            normalization_min=normalization_min, fix_probe_com=fix_probe_com,
            fix_probe=fix_probe, fix_positions=fix_positions,
            fix_positions_com=fix_positions_com, positions_step_size=positions_step_size,
            max_position_update_distance=max_position_update_distance,
            max_position_total_distance=max_position_total_distance,
            pure_phase_object=pure_phase_object, object_positivity=object_positivity,
            shrinkage_rad=shrinkage_rad, fix_potential_baseline=fix_potential_baseline,
            detector_fourier_mask=detector_fourier_mask, store_iterations=store_iterations,
            reset=reset, device=device, clear_fft_cache=clear_fft_cache,
            object_type=object_type, orthogonalize_probe=orthogonalize_probe,
            fix_probe_aperture=fix_probe_aperture and not fix_probe,
            constrain_probe_amplitude=constrain_probe_amplitude and not fix_probe,
            constrain_probe_amplitude_relative_radius=constrain_probe_amplitude_relative_radius,
            constrain_probe_amplitude_relative_width=constrain_probe_amplitude_relative_width,
            gaussian_filter_sigma=gaussian_filter_sigma if gaussian_filter else None,
            global_affine_transformation=global_affine_transformation and not fix_positions,
            unsupported=dict(
                constrain_probe_fourier_amplitude=constrain_probe_fourier_amplitude
                and not fix_probe,
                fit_probe_aberrations=fit_probe_aberrations and not fix_probe,
                butterworth_filter=butterworth_filter
                and (q_lowpass is not None or q_highpass is not None),
                tv_denoise=tv_denoise and tv_denoise_weight is not None,
            ))


class MultislicePtychography(_PtychographyBase):
    """Multislice ptychography (object (T,Px,Py), Fresnel propagation between slices)."""

    _multislice = True

    def __init__(
        self,
        energy: float,
        num_slices: int,
        slice_thicknesses: Union[float, Sequence[float]],
        datacube=None,
        semiangle_cutoff: float = None,
        semiangle_cutoff_pixels: float = None,
        rolloff: float = 2.0,
        vacuum_probe_intensity: np.ndarray = None,
        polar_parameters: Mapping[str, float] = None,
        object_padding_px: Tuple[int, int] = None,
        initial_object_guess: np.ndarray = None,
        initial_probe_guess: np.ndarray = None,
        initial_scan_positions: np.ndarray = None,
        object_fov_ang: Tuple[float, float] = None,
        positions_offset_ang: np.ndarray = None,
        theta_x: float = None,
        theta_y: float = None,
        middle_focus: bool = False,
        object_type: str = "complex",
        positions_mask: np.ndarray = None,
        verbose: bool = True,
        device: str = "gpu",
        storage: str = None,
        clear_fft_cache: bool = True,
        name: str = "multi-slice_ptychographic_reconstruction",
        **kwargs,
    ):
        slice_thicknesses = np.array(slice_thicknesses)
        if slice_thicknesses.shape == ():
            slice_thicknesses = np.tile(slice_thicknesses, num_slices - 1)
        elif slice_thicknesses.shape[0] != (num_slices - 1):
            raise ValueError(
                f"slice_thicknesses must have length {num_slices - 1}, "
                f"not {slice_thicknesses.shape[0]}.")
        self._common_init(energy, datacube, semiangle_cutoff, semiangle_cutoff_pixels, rolloff,
                          vacuum_probe_intensity, polar_parameters, initial_object_guess,
                          initial_probe_guess, initial_scan_positions, object_fov_ang,
                          positions_offset_ang, object_padding_px, object_type, positions_mask,
                          verbose, device, storage, clear_fft_cache, name, kwargs)
        if middle_focus:
            half = slice_thicknesses.mean() * num_slices / 2
            self._polar_parameters["C10"] -= half
        self._num_slices = num_slices
        self._slice_thicknesses = slice_thicknesses
        self._theta_x = theta_x
        self._theta_y = theta_y

    preprocess = SingleslicePtychography.preprocess

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
        kz_regularization_filter: bool = True,
        kz_regularization_gamma: float = None,
        identical_slices: bool = False,
        object_positivity: bool = True,
        shrinkage_rad: float = 0.0,
        fix_potential_baseline: bool = True,
        detector_fourier_mask: np.ndarray = None,
        pure_phase_object: bool = False,
        tv_denoise_chambolle: bool = True,
        tv_denoise_weight_chambolle=None,
        tv_denoise_pad_chambolle=1,
        tv_denoise: bool = True,
        tv_denoise_weights=None,
        tv_denoise_inner_iter=40,
        store_iterations: bool = False,
        progress_bar: bool = True,
        reset: bool = None,
        device: str = None,
        clear_fft_cache: bool = None,
        object_type: str = None,
    ):
        """Run `num_iter` multislice iterations on the GPU."""
        return self._reconstruct_impl(
            num_iter=num_iter, reconstruction_method=reconstruction_method,
            reconstruction_parameter=reconstruction_parameter,
            reconstruction_parameter_a=reconstruction_parameter_a,
            reconstruction_parameter_b=reconstruction_parameter_b,
            reconstruction_parameter_c=reconstruction_parameter_c,
            max_batch_size=max_batch_size, seed_random=seed_random, step_size=step_size,
            normalization_min=normalization_min, fix_probe_com=fix_probe_com,
            fix_probe=fix_probe, fix_positions=fix_positions,
            fix_positions_com=fix_positions_com, positions_step_size=positions_step_size,
            max_position_update_distance=max_position_update_distance,
            max_position_total_distance=max_position_total_distance,
            pure_phase_object=pure_phase_object, object_positivity=object_positivity,
            shrinkage_rad=shrinkage_rad, fix_potential_baseline=fix_potential_baseline,
            detector_fourier_mask=detector_fourier_mask, store_iterations=store_iterations,
            reset=reset, device=device, clear_fft_cache=clear_fft_cache,
            object_type=object_type,
            fix_probe_aperture=fix_probe_aperture and not fix_probe,
            constrain_probe_amplitude=constrain_probe_amplitude and not fix_probe,
            constrain_probe_amplitude_relative_radius=constrain_probe_amplitude_relative_radius,
            constrain_probe_amplitude_relative_width=constrain_probe_amplitude_relative_width,
            gaussian_filter_sigma=gaussian_filter_sigma if gaussian_filter else None,
            identical_slices=identical_slices,
            global_affine_transformation=global_affine_transformation and not fix_positions,
            unsupported=dict(
                constrain_probe_fourier_amplitude=constrain_probe_fourier_amplitude
                and not fix_probe,
                fit_probe_aberrations=fit_probe_aberrations and not fix_probe,
                butterworth_filter=butterworth_filter
                and (q_lowpass is not None or q_highpass is not None),
                kz_regularization_filter=kz_regularization_filter
                and kz_regularization_gamma is not None,
                tv_denoise=tv_denoise and tv_denoise_weights is not None,
                tv_denoise_chambolle=tv_denoise_chambolle
                and tv_denoise_weight_chambolle is not None,
            ))


class MixedstateMultislicePtychography(_PtychographyBase):
    """Mixed-state multislice ptychography: object (T,Px,Py), probe (M,Sx,Sy)
    incoherent modes, each propagated through the slices
    (mixedstate_multislice_ptychography.py; operators
    ptychographic_methods.py:3096-3400)."""

    _multislice = True
    _mixed = True

    def __init__(
        self,
        energy: float,
        num_slices: int,
        slice_thicknesses: Union[float, Sequence[float]],
        num_probes: int = None,
        datacube=None,
        semiangle_cutoff: float = None,
        semiangle_cutoff_pixels: float = None,
        rolloff: float = 2.0,
        vacuum_probe_intensity: np.ndarray = None,
        polar_parameters: Mapping[str, float] = None,
        object_padding_px: Tuple[int, int] = None,
        initial_object_guess: np.ndarray = None,
        initial_probe_guess: np.ndarray = None,
        initial_scan_positions: np.ndarray = None,
        object_fov_ang: Tuple[float, float] = None,
        positions_offset_ang: np.ndarray = None,
        theta_x: float = 0,
        theta_y: float = 0,
        middle_focus: bool = False,
        object_type: str = "complex",
        positions_mask: np.ndarray = None,
        verbose: bool = True,
        device: str = "gpu",
        storage: str = None,
        clear_fft_cache: bool = True,
        name: str = "multi-slice_ptychographic_reconstruction",
        **kwargs,
    ):
        if initial_probe_guess is None or isinstance(initial_probe_guess, ComplexProbe):
            if num_probes is None:
                raise ValueError(
                    "If initial_probe_guess is None, or a ComplexProbe object, "
                    "num_probes must be specified.")
        else:
            if len(initial_probe_guess.shape) != 3:
                raise ValueError("Specified initial_probe_guess must have dimensions (N,Sx,Sy).")
            num_probes = initial_probe_guess.shape[0]
        slice_thicknesses = np.array(slice_thicknesses)
        if slice_thicknesses.shape == ():
            slice_thicknesses = np.tile(slice_thicknesses, num_slices - 1)
        elif slice_thicknesses.shape[0] != (num_slices - 1):
            raise ValueError(
                f"slice_thicknesses must have length {num_slices - 1}, "
                f"not {slice_thicknesses.shape[0]}.")
        self._common_init(energy, datacube, semiangle_cutoff, semiangle_cutoff_pixels, rolloff,
                          vacuum_probe_intensity, polar_parameters, initial_object_guess,
                          initial_probe_guess, initial_scan_positions, object_fov_ang,
                          positions_offset_ang, object_padding_px, object_type, positions_mask,
                          verbose, device, storage, clear_fft_cache, name, kwargs)
        if middle_focus:
            half = slice_thicknesses.mean() * num_slices / 2
            self._polar_parameters["C10"] -= half
        self._num_probes = num_probes
        self._num_slices = num_slices
        self._slice_thicknesses = slice_thicknesses
        self._theta_x = theta_x
        self._theta_y = theta_y

    preprocess = SingleslicePtychography.preprocess

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
        orthogonalize_probe: bool = True,
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
        num_probes_fit_aberrations: int = np.inf,
        butterworth_filter: bool = True,
        q_lowpass: float = None,
        q_highpass: float = None,
        butterworth_order: float = 2,
        kz_regularization_filter: bool = True,
        kz_regularization_gamma: Union[float, np.ndarray] = None,
        identical_slices: bool = False,
        object_positivity: bool = True,
        shrinkage_rad: float = 0.0,
        fix_potential_baseline: bool = True,
        detector_fourier_mask: np.ndarray = None,
        pure_phase_object: bool = False,
        tv_denoise_chambolle: bool = True,
        tv_denoise_weight_chambolle=None,
        tv_denoise_pad_chambolle=1,
        tv_denoise: bool = True,
        tv_denoise_weights=None,
        tv_denoise_inner_iter=40,
        store_iterations: bool = False,
        progress_bar: bool = True,
        reset: bool = None,
        device: str = None,
        clear_fft_cache: bool = None,
        object_type: str = None,
    ):
        """Run `num_iter` mixed-state multislice iterations on the GPU
        (mixedstate_multislice_ptychography.py:723-1146)."""
        return self._reconstruct_impl(
            num_iter=num_iter, reconstruction_method=reconstruction_method,
            reconstruction_parameter=reconstruction_parameter,
            reconstruction_parameter_a=reconstruction_parameter_a,
            reconstruction_parameter_b=reconstruction_parameter_b,
            reconstruction_parameter_c=reconstruction_parameter_c,
            max_batch_size=max_batch_size, seed_random=seed_random, step_size=step_size,
            normalization_min=normalization_min, fix_probe_com=fix_probe_com,
            fix_probe=fix_probe, fix_positions=fix_positions,
            fix_positions_com=fix_positions_com, positions_step_size=positions_step_size,
            max_position_update_distance=max_position_update_distance,
            max_position_total_distance=max_position_total_distance,
            pure_phase_object=pure_phase_object, object_positivity=object_positivity,
            shrinkage_rad=shrinkage_rad, fix_potential_baseline=fix_potential_baseline,
            detector_fourier_mask=detector_fourier_mask, store_iterations=store_iterations,
            reset=reset, device=device, clear_fft_cache=clear_fft_cache,
            object_type=object_type, orthogonalize_probe=orthogonalize_probe,
            fix_probe_aperture=fix_probe_aperture and not fix_probe,
            constrain_probe_amplitude=constrain_probe_amplitude and not fix_probe,
            constrain_probe_amplitude_relative_radius=constrain_probe_amplitude_relative_radius,
            constrain_probe_amplitude_relative_width=constrain_probe_amplitude_relative_width,
            gaussian_filter_sigma=gaussian_filter_sigma if gaussian_filter else None,
            identical_slices=identical_slices,
            global_affine_transformation=global_affine_transformation and not fix_positions,
            unsupported=dict(
                constrain_probe_fourier_amplitude=constrain_probe_fourier_amplitude
                and not fix_probe,
                fit_probe_aberrations=fit_probe_aberrations and not fix_probe,
                butterworth_filter=butterworth_filter
                and (q_lowpass is not None or q_highpass is not None),
                kz_regularization_filter=kz_regularization_filter
                and kz_regularization_gamma is not None,
                tv_denoise=tv_denoise and tv_denoise_weights is not None,
                tv_denoise_chambolle=tv_denoise_chambolle
                and tv_denoise_weight_chambolle is not None,
            ))
