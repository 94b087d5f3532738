"""Load the golden fixtures written by tests/golden/make_golden.py."""

import glob
import json
import os

import numpy as np

from py4dstem_gb300 import DataCube
from py4dstem_gb300 import ptychography as api
from oracle.ptycho_np import State

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _all_names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def names():
    """Reconstruction fixtures of the 2D / multislice / mixed-state classes
    (the tomography fixtures, tomo_*, and the fixtures at the timed sizes,
    size_*, which keep no datacube, have their own tests)."""
    return [n for n in _all_names() if not n.startswith(("prep_", "tomo_", "size_"))]


def prep_names():
    """Preprocess-only fixtures."""
    return [n for n in _all_names() if n.startswith("prep_")]


class PrepGolden:
    """A preprocess-only fixture: datacube, options and the reference's
    preprocessed state."""

    def __init__(self, name):
        self.name = name
        z = np.load(os.path.join(GOLDEN_DIR, f"{name}.npz"))
        self.meta = json.loads(str(z["meta"]))
        self.datacube_counts = z["datacube"].astype(np.float32)
        self.scan_positions_ang = z["scan_positions_ang"]
        self.positions_mask = z["positions_mask"] if "positions_mask" in z.files else None
        self.dp_mask = z["dp_mask"] if "dp_mask" in z.files else None
        self.vacuum = (z["vacuum_probe_intensity"] if "vacuum_probe_intensity" in z.files
                       else None)
        self.pre = {k[4:]: z[k] for k in z.files if k.startswith("pre_")}

    def build(self, device="gpu", storage=None):
        m = self.meta
        ctor = dict(m["ctor"])
        if "object_fov_ang" in ctor:
            ctor["object_fov_ang"] = tuple(ctor["object_fov_ang"])
        kw = {}
        if m["scan_positions"]:
            kw["initial_scan_positions"] = self.scan_positions_ang.copy()
        if self.positions_mask is not None:
            kw["positions_mask"] = self.positions_mask.copy()
        if self.vacuum is not None:
            kw["vacuum_probe_intensity"] = self.vacuum.copy()
        dc = DataCube(self.datacube_counts.copy(), r_pixel_size=m["r_pixel_size"],
                      r_pixel_units="A", q_pixel_size=m["q_pixel_size"], q_pixel_units="mrad")
        p = api.SingleslicePtychography(datacube=dc, verbose=False, device=device,
                                        storage=storage, **ctor, **kw)
        pre = dict(m["preprocess"])
        if self.dp_mask is not None:
            pre["dp_mask"] = self.dp_mask.copy()
        p.preprocess(**pre)
        return p

    @staticmethod
    def same_state(p, q):
        """Assert that two preprocessed objects hold the same bits."""
        for key in ("com_measured_x", "com_measured_y", "com_fitted_x", "com_fitted_y",
                    "com_normalized_x", "com_normalized_y", "positions_px", "probe",
                    "object_fov_mask"):
            a, b = np.asarray(getattr(p, "_" + key)), np.asarray(getattr(q, "_" + key))
            assert a.dtype == b.dtype, key
            np.testing.assert_array_equal(a, b, err_msg=key)
        assert p._rotation_best_rad == q._rotation_best_rad
        assert p._rotation_best_transpose == q._rotation_best_transpose
        assert np.float32(p._mean_diffraction_intensity) == np.float32(q._mean_diffraction_intensity)
        np.testing.assert_array_equal(p._amplitudes, q._amplitudes)

    def check(self, p, fov_mask=True, probe_exact=True):
        """Assert that a preprocessed object holds the reference's bits. The
        initial probe is NumPy FFT work on the host, whose float32 bits may differ
        between CPU architectures for sizes that are not powers of two:
        probe_exact=False compares it to 1e-6."""
        r = self.pre
        for key in ("com_measured_x", "com_measured_y", "com_fitted_x", "com_fitted_y",
                    "com_normalized_x", "com_normalized_y"):
            np.testing.assert_array_equal(np.asarray(getattr(p, "_" + key)), r[key], err_msg=key)
        assert np.float64(p._rotation_best_rad) == r["rotation_best_rad"]
        assert bool(p._rotation_best_transpose) == bool(r["rotation_best_transpose"])
        assert np.float32(p._mean_diffraction_intensity) == r["mean_intensity"]
        np.testing.assert_array_equal(p._positions_px, r["positions_px"])
        if probe_exact:
            np.testing.assert_array_equal(p._probe, r["probe_initial"])
        else:
            assert rel_l2(p._probe, r["probe_initial"]) < 1e-6
        np.testing.assert_array_equal(p._amplitudes, r["amplitudes"])
        if fov_mask:
            np.testing.assert_array_equal(p._object_fov_mask, r["fov_mask"])


class Golden:
    def __init__(self, name):
        self.name = name
        z = np.load(os.path.join(GOLDEN_DIR, f"{name}.npz"))
        self.meta = json.loads(str(z["meta"]))
        self.datacube_counts = z["datacube"].astype(np.float32)
        self.scan_positions_ang = z["scan_positions_ang"]
        self.pre = {k[4:]: z[k] for k in z.files if k.startswith("pre_")}
        self.out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
        self.guess = z["initial_object_guess"] if "initial_object_guess" in z.files else None
        self.mask = z["detector_fourier_mask"] if "detector_fourier_mask" in z.files else None

    def rec_kwargs(self):
        """reconstruct() arguments of the fixture (the detector mask included)."""
        r = dict(self.meta["reconstruct"])
        if self.mask is not None:
            r["detector_fourier_mask"] = self.mask.copy()
        return r

    @property
    def projection(self):
        return self.meta["reconstruct"].get("reconstruction_method", "GD") not in (
            "GD", "gradient-descent")

    def datacube(self):
        return DataCube(self.datacube_counts.copy(), r_pixel_size=self.meta["r_pixel_size"],
                        r_pixel_units="A", q_pixel_size=self.meta["q_pixel_size"],
                        q_pixel_units="mrad")

    def build(self, device="gpu", storage=None):
        """Construct and preprocess the product class exactly as the reference was."""
        m = self.meta
        ctor = dict(m["ctor"])
        if "object_fov_ang" in ctor:
            ctor["object_fov_ang"] = tuple(ctor["object_fov_ang"])
        cls = {"single": api.SingleslicePtychography, "multi": api.MultislicePtychography,
               "mixed": api.MixedstatePtychography,
               "mixed_multi": api.MixedstateMultislicePtychography}[m["cls"]]
        if self.guess is not None:
            ctor["initial_object_guess"] = self.guess.copy()
        if m.get("global_seed") is not None:
            np.random.seed(m["global_seed"])
        p = cls(datacube=self.datacube(), initial_scan_positions=self.scan_positions_ang.copy(),
                verbose=False, device=device, storage=storage, **ctor)
        p.preprocess(**m["preprocess"])
        return p

    def state(self, p):
        """Oracle state from a preprocessed product object."""
        m = self.meta
        return State(
            amplitudes=p._amplitudes, positions_px=p._positions_px.copy(),
            probe=np.array(p._probe, copy=True), object=np.array(p._object, copy=True),
            mean_intensity=p._mean_diffraction_intensity,
            fov_mask_inverse=p._object_fov_mask_inverse, object_type=p._object_type,
            num_slices=m["ctor"].get("num_slices", 1), num_probes=m["ctor"].get("num_probes", 1),
            mixed=m["cls"] in ("mixed", "mixed_multi"),
            propagators=(getattr(p, "_propagator_arrays", None)
                         if m["cls"] in ("multi", "mixed_multi") else None),
            sampling=tuple(p.sampling),
            roi_shape=tuple(int(v) for v in p._region_of_interest_shape),
            resample_exit_waves=bool(getattr(p, "_resample_exit_waves", False)))

    def oracle_kwargs(self):
        from oracle.ptycho_np import method_abc

        r = self.rec_kwargs()
        method, a, b, c = method_abc(r.pop("reconstruction_method", "GD"),
                                     r.pop("reconstruction_parameter", 1.0))
        return dict(method=method, a=a, b=b, c=c, **r)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
