"""Saving and reading a reconstruction.

The reference writes a reconstruction to an emdfile/HDF5 tree
(phase_base_class.py:1526-1665, ``to_h5``) and reads it back by constructing the
class from the stored instantiation metadata and filling in the preprocessing
metadata (``_get_constructor_args`` / ``_populate_instance``,
phase_base_class.py:1667-1763). h5py and emdfile are not part of this package,
so the same content goes into one NumPy ``.npz`` file: the arrays as entries and
the metadata as a JSON string.

Content, as the reference stores it:

* instantiation metadata: energy, semiangle cutoff, rolloff, object padding,
  object field of view, object type, name, vacuum probe, the scan positions
  (the pixel positions times the sampling, rotated back by the best-fit
  rotation about their mean) and each class's own constructor values
  (slices, slice thicknesses, tilts, probe modes);
* the polar aberration coefficients;
* preprocessing metadata: rotation angle and transpose, pixel positions,
  region-of-interest and amplitude shapes, pattern count, angular sampling,
  positions mask;
* the error history, the object and the probe; the iteration snapshots (every
  ``save_iterations_frequency``-th) when ``save_iterations``; the exit waves when
  ``save_exit_waves``; the datacube and its calibration when ``save_datacube``
  (``set_save_defaults``).

Reading constructs the class with the stored object and probe as the initial
guesses and marks it preprocessed, like the reference; to continue
reconstructing, attach the datacube (or save it) and call ``preprocess()``.

``PtychographicTomography`` stores the same kinds of content for its volume and
its tilts: the tilt orientation matrices, every tilt's scan positions (rotated
back, concatenated, with the cumulative pattern counts), the per-tilt mean
intensities and probes, the volume, the slice thicknesses, and each tilt's
datacube when ``save_datacube``.
"""

from __future__ import annotations

import json

import numpy as np

from .datacube import DataCube
from .preprocess import rotate_positions

_CLASS_SPECIFIC = {
    "SingleslicePtychography": (),
    "MixedstatePtychography": ("_num_probes",),
    "MultislicePtychography": ("_num_slices", "_slice_thicknesses", "_theta_x", "_theta_y"),
    "MixedstateMultislicePtychography": ("_num_probes", "_num_slices", "_slice_thicknesses",
                                         "_theta_x", "_theta_y"),
}


def _jsonable(v):
    if isinstance(v, np.ndarray):
        return {"__array__": v.tolist(), "dtype": str(v.dtype)}
    if isinstance(v, (np.floating, np.integer, np.bool_)):
        return v.item()
    if isinstance(v, (tuple, list)):
        return [_jsonable(x) for x in v]
    if isinstance(v, dict):
        return {k: _jsonable(x) for k, x in v.items()}
    return v


def _unjson(v):
    if isinstance(v, dict) and "__array__" in v:
        return np.asarray(v["__array__"], dtype=v["dtype"])
    if isinstance(v, dict):
        return {k: _unjson(x) for k, x in v.items()}
    if isinstance(v, list):
        return [_unjson(x) for x in v]
    return v


def _calibration(dc):
    c = dc.calibration
    return {"R_pixel_size": c.get_R_pixel_size(), "R_pixel_units": c.get_R_pixel_units(),
            "Q_pixel_size": c.get_Q_pixel_size(), "Q_pixel_units": c.get_Q_pixel_units()}


def _datacube(data, c):
    return DataCube(data, r_pixel_size=c["R_pixel_size"], r_pixel_units=c["R_pixel_units"],
                    q_pixel_size=c["Q_pixel_size"], q_pixel_units=c["Q_pixel_units"])


def _save_tomography(path, p) -> None:
    arrays = {}
    rot = p._rotation_best_rad
    cum = np.asarray(p._cum_probes_per_measurement)
    pos = np.asarray(p._positions_initial_all, dtype=np.float64)
    arrays["scan_positions"] = rotate_positions(pos, -rot) if rot is not None else pos
    arrays["cum_probes_per_measurement"] = cum
    arrays["tilt_orientation_matrices"] = np.stack(
        [np.asarray(m, dtype=np.float64) for m in p._tilt_orientation_matrices])
    if p._vacuum_probe_intensity is not None:
        arrays["vacuum_probe_intensity"] = np.asarray(p._vacuum_probe_intensity)
    arrays["positions_px"] = np.asarray(p._positions_px_all)
    arrays["object"] = np.asarray(p._object)
    arrays["probes"] = np.stack([np.asarray(pr) for pr in p._probes_all])
    arrays["mean_intensity"] = np.asarray(p._mean_diffraction_intensity, dtype=np.float32)
    arrays["slice_thicknesses"] = np.asarray(p._slice_thicknesses)
    instantiation = {
        "energy": p._energy, "num_slices": p._num_slices,
        "semiangle_cutoff": p._semiangle_cutoff, "rolloff": p._rolloff,
        "object_padding_px": p._object_padding_px, "object_type": p._object_type,
        "verbose": p._verbose, "device": p._device, "storage": p._storage,
        "clear_fft_cache": getattr(p, "_clear_fft_cache", True), "name": p.name,
    }
    preprocess = {
        "rotation_angle_rad": rot, "data_transpose": p._rotation_best_transpose,
        "region_of_interest_shape": np.asarray(p._region_of_interest_shape),
        "amplitudes_shape": np.asarray(p._amplitudes_shape),
        "num_diffraction_patterns": int(p._num_diffraction_patterns),
        "angular_sampling": p.angular_sampling,
    }
    if p._save_iterations and getattr(p, "object_iterations", None):
        every = range(0, len(p.object_iterations), p._save_iterations_frequency)
        arrays["object_iterations"] = np.stack([np.asarray(p.object_iterations[i])
                                                for i in every])
        arrays["probe_iterations"] = np.stack([np.stack(p.probe_iterations[i]) for i in every])
    calibrations = None
    if p._save_datacube and p._datacube is not None:
        calibrations = []
        for i, dc in enumerate(p._datacube):
            arrays[f"datacube_{i}"] = np.asarray(dc.data)
            calibrations.append(_calibration(dc))
    meta = {
        "class": "PtychographicTomography",
        "instantiation_metadata": instantiation,
        "aberrations_metadata": dict(p._polar_parameters),
        "preprocess_metadata": preprocess,
        "reconstruction_metadata": {
            "reconstruction_error": list(getattr(p, "error_iterations", []))},
        "calibration": calibrations,
    }
    np.savez(path, meta=json.dumps(_jsonable(meta)), **arrays)


def _read_tomography(z, meta, device, storage, verbose):
    from .tomography import PtychographicTomography

    inst = meta["instantiation_metadata"]
    cum = np.asarray(z["cum_probes_per_measurement"])
    n_meas = len(cum) - 1
    scan = np.asarray(z["scan_positions"])
    datacube = None
    if meta["calibration"] is not None:
        datacube = [_datacube(z[f"datacube_{i}"], c) for i, c in enumerate(meta["calibration"])]
    probes = [np.asarray(pr) for pr in z["probes"]]
    p = PtychographicTomography(
        energy=inst["energy"], num_slices=inst["num_slices"],
        tilt_orientation_matrices=list(z["tilt_orientation_matrices"]), datacube=datacube,
        semiangle_cutoff=inst["semiangle_cutoff"], rolloff=inst["rolloff"],
        vacuum_probe_intensity=(np.asarray(z["vacuum_probe_intensity"])
                                if "vacuum_probe_intensity" in z.files else None),
        polar_parameters=dict(meta["aberrations_metadata"]),
        object_padding_px=inst["object_padding_px"], object_type=inst["object_type"],
        initial_object_guess=np.asarray(z["object"]), initial_probe_guess=probes,
        initial_scan_positions=[scan[cum[i]:cum[i + 1]] for i in range(n_meas)],
        name=inst["name"], verbose=verbose, device=device,
        storage=storage if storage is not None else device)
    pre = meta["preprocess_metadata"]
    p._rotation_best_rad = pre["rotation_angle_rad"]
    p._rotation_best_transpose = pre["data_transpose"]
    p._angular_sampling = tuple(pre["angular_sampling"])
    p._region_of_interest_shape = np.asarray(pre["region_of_interest_shape"])
    p._amplitudes_shape = np.asarray(pre["amplitudes_shape"])
    p._num_diffraction_patterns = pre["num_diffraction_patterns"]
    p._cum_probes_per_measurement = cum
    p._positions_px_all = np.asarray(z["positions_px"])
    p._positions_px_initial_all = p._positions_px_all.copy()
    p._mean_diffraction_intensity = [np.float32(v) for v in z["mean_intensity"]]
    p._object = np.asarray(z["object"])
    p._object_initial = p._object.copy()
    p._object_type_initial = p._object_type
    p._object_shape = p._object.shape[-2:]
    p._num_voxels = p._object.shape[0]
    p._probes_all = [pr.copy() for pr in probes]
    p._probes_all_initial = [pr.copy() for pr in probes]
    p._slice_thicknesses = np.asarray(z["slice_thicknesses"])
    p._propagator_arrays = p._fresnel_propagators()
    p._object_fov_mask = np.full(p._object_shape, True)
    p._object_fov_mask_inverse = np.invert(p._object_fov_mask)
    if "object_iterations" in z.files:
        p.object_iterations = list(z["object_iterations"])
        p.probe_iterations = [list(pr) for pr in z["probe_iterations"]]
    error = list(meta["reconstruction_metadata"]["reconstruction_error"])
    p.error_iterations = error
    if error:
        p.error = error[-1]
    p.object = p._object.copy()
    p.probe = p.probe_centered
    p._preprocessed = True
    return p


def save(path, ptycho) -> None:
    """Write a preprocessed (and possibly reconstructed) object to `path` (.npz)."""
    cls = type(ptycho).__name__
    if cls == "PtychographicTomography":
        if not getattr(ptycho, "_preprocessed", False):
            raise ValueError("preprocess() the object before saving it")
        return _save_tomography(path, ptycho)
    if cls not in _CLASS_SPECIFIC:
        raise TypeError(f"cannot save a {cls}")
    if not getattr(ptycho, "_preprocessed", False):
        raise ValueError("preprocess() the object before saving it")
    arrays = {}
    rot = ptycho._rotation_best_rad
    pos = ptycho.positions
    scan_positions = rotate_positions(pos, -rot) if rot is not None else pos
    vpi = ptycho._vacuum_probe_intensity
    if vpi is not None:
        arrays["vacuum_probe_intensity"] = np.asarray(vpi)
    instantiation = {
        "energy": ptycho._energy,
        "semiangle_cutoff": ptycho._semiangle_cutoff,
        "rolloff": ptycho._rolloff,
        "object_padding_px": ptycho._object_padding_px,
        "object_fov_ang": ptycho._object_fov_ang,
        "object_type": ptycho._object_type,
        "verbose": ptycho._verbose,
        "device": ptycho._device,
        "storage": ptycho._storage,
        "clear_fft_cache": getattr(ptycho, "_clear_fft_cache", True),
        "name": ptycho.name,
    }
    for key in _CLASS_SPECIFIC[cls]:
        instantiation[key[1:]] = getattr(ptycho, key, None)
    arrays["scan_positions"] = np.asarray(scan_positions)
    pmask = ptycho._positions_mask
    if pmask is not None and np.ndim(pmask) > 0 and pmask[0] is not None:
        arrays["positions_mask"] = np.asarray(pmask)
    preprocess = {
        "rotation_angle_rad": rot,
        "data_transpose": ptycho._rotation_best_transpose,
        "region_of_interest_shape": np.asarray(ptycho._region_of_interest_shape),
        "amplitudes_shape": np.asarray(ptycho._amplitudes_shape),
        "num_diffraction_patterns": ptycho._num_diffraction_patterns,
        "sampling": ptycho.sampling,
        "angular_sampling": ptycho.angular_sampling,
    }
    arrays["positions_px"] = np.asarray(ptycho._positions_px)
    arrays["object"] = np.asarray(ptycho._object)
    arrays["probe"] = np.asarray(ptycho._probe)
    error = list(getattr(ptycho, "error_iterations", []))
    if ptycho._save_iterations and hasattr(ptycho, "object_iterations"):
        every = range(0, len(ptycho.object_iterations), ptycho._save_iterations_frequency)
        arrays["object_iterations"] = np.stack([np.asarray(ptycho.object_iterations[i])
                                                for i in every])
        arrays["probe_iterations"] = np.stack([np.asarray(ptycho.probe_iterations[i])
                                               for i in every])
    if ptycho._save_exit_waves and ptycho._exit_waves is not None:
        arrays["exit_waves"] = np.asarray(ptycho._exit_waves)
    calibration = None
    if ptycho._save_datacube and ptycho._datacube is not None:
        dc = ptycho._datacube
        arrays["datacube"] = np.asarray(dc.data)
        c = dc.calibration
        calibration = {"R_pixel_size": c.get_R_pixel_size(), "R_pixel_units": c.get_R_pixel_units(),
                       "Q_pixel_size": c.get_Q_pixel_size(), "Q_pixel_units": c.get_Q_pixel_units()}
    meta = {
        "class": cls,
        "instantiation_metadata": instantiation,
        "aberrations_metadata": dict(ptycho._polar_parameters),
        "preprocess_metadata": preprocess,
        "reconstruction_metadata": {"reconstruction_error": error},
        "calibration": calibration,
    }
    np.savez(path, meta=json.dumps(_jsonable(meta)), **arrays)


def read(path, device: str = "gpu", storage: str = None, verbose: bool = True):
    """Construct the saved class from `path`, with the saved object and probe as
    initial guesses and the preprocessing metadata filled in."""
    from . import ptychography

    z = np.load(path, allow_pickle=False)
    meta = _unjson(json.loads(str(z["meta"])))
    if meta["class"] == "PtychographicTomography":
        return _read_tomography(z, meta, device, storage, verbose)
    cls = getattr(ptychography, meta["class"])
    inst = meta["instantiation_metadata"]
    datacube = None
    if "datacube" in z.files and meta["calibration"] is not None:
        c = meta["calibration"]
        datacube = DataCube(z["datacube"], r_pixel_size=c["R_pixel_size"],
                            r_pixel_units=c["R_pixel_units"], q_pixel_size=c["Q_pixel_size"],
                            q_pixel_units=c["Q_pixel_units"])
    kwargs = dict(
        datacube=datacube,
        initial_object_guess=np.asarray(z["object"]),
        initial_probe_guess=np.asarray(z["probe"]),
        vacuum_probe_intensity=(np.asarray(z["vacuum_probe_intensity"])
                                if "vacuum_probe_intensity" in z.files else None),
        initial_scan_positions=np.asarray(z["scan_positions"]),
        energy=inst["energy"],
        object_padding_px=inst["object_padding_px"],
        object_type=inst["object_type"],
        semiangle_cutoff=inst["semiangle_cutoff"],
        rolloff=inst["rolloff"],
        name=inst["name"],
        polar_parameters=dict(meta["aberrations_metadata"]),
        verbose=verbose,
        device=device,
        storage=storage if storage is not None else device,
    )
    for key in _CLASS_SPECIFIC[meta["class"]]:
        value = inst[key[1:]]
        if key == "_slice_thicknesses":
            value = np.asarray(value)
        kwargs[key[1:]] = value
    p = cls(**kwargs)
    pre = meta["preprocess_metadata"]
    p._rotation_best_rad = pre["rotation_angle_rad"]
    p._rotation_best_transpose = pre["data_transpose"]
    p._positions_px = np.asarray(z["positions_px"])
    p._angular_sampling = tuple(pre["angular_sampling"])
    p._region_of_interest_shape = np.asarray(pre["region_of_interest_shape"])
    p._amplitudes_shape = np.asarray(pre["amplitudes_shape"])
    p._num_diffraction_patterns = pre["num_diffraction_patterns"]
    p._positions_mask = np.asarray(z["positions_mask"]) if "positions_mask" in z.files else None
    p._exit_waves = (np.asarray(z["exit_waves"], dtype=np.complex64)
                     if "exit_waves" in z.files else None)
    if "object_iterations" in z.files:
        p.object_iterations = list(z["object_iterations"])
        p.probe_iterations = list(z["probe_iterations"])
    error = list(meta["reconstruction_metadata"]["reconstruction_error"])
    p.error_iterations = error
    if error:
        p.error = error[-1]
    p._positions_px_com = np.mean(p._positions_px, axis=0)
    p._object = np.asarray(z["object"])
    p._probe = np.asarray(z["probe"])
    p.object = np.asarray(p._object)
    p.probe = p.probe_centered
    p._preprocessed = True
    return p
