"""Tomography oracle and host side, no GPU.

* The restated volume operations (oracle/tomography_np.py) against the
  reference's own _rotate_zxy_volume, _project_sliced_object and
  _expand_sliced_object outputs (tests/golden/tomo_volume_ops.npz) and against
  SciPy on edge shapes.
* The host preprocess() of py4dstem_gb300.PtychographicTomography against the
  reference's preprocessed state (tests/golden/tomo_*.npz).
* The oracle's reconstruction loop against the reference's result.
* Options without a GPU implementation raise before any device work.
"""

import json
import os

import numpy as np
import pytest

from oracle import tomography_np as tomo

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
TOMO_CASES = ("tomo_gd_collective", "tomo_gd_sequential", "tomo_gd_zero_start",
              "tomo_gd_gaussian")


def _ops():
    return np.load(os.path.join(GOLDEN, "tomo_volume_ops.npz"))


def test_rotation_matches_reference():
    z = _ops()
    for k in range(4):
        m = z[f"matrix_{k}"]
        out = tomo.rotate_volume(z["volume"], m)
        assert out.dtype == np.float32
        assert np.array_equal(out, z[f"rot32_{k}"])
        out64 = tomo.rotate_volume(z["volume64"], m)
        assert out64.dtype == np.float64
        assert np.abs(out64 - z[f"rot64_{k}"]).max() < 1e-13


def test_project_and_expand_match_reference():
    z = _ops()
    for t in (1, 3, 6, 7):
        assert np.array_equal(tomo.project_sliced(z["volume"], t), z[f"project_{t}"])
        e = tomo.expand_sliced(z[f"update_{t}"], z["volume"].shape[0])
        assert e.dtype == np.float64 and np.array_equal(e, z[f"expand_{t}"])


@pytest.mark.parametrize("shape", [(1, 5, 7), (2, 3, 4), (5, 1, 6), (6, 6, 2)])
def test_rotation_edge_shapes_match_scipy(shape):
    from scipy.ndimage import affine_transform

    rng = np.random.default_rng(sum(shape))
    vol = rng.random(shape).astype(np.float32)
    t = np.deg2rad(23.0)
    rot = np.array([[1, 0, 0], [0, np.cos(t), -np.sin(t)], [0, np.sin(t), np.cos(t)]])
    tf, off = tomo.rotation_transform(shape, rot)
    ref = affine_transform(vol, tf, offset=off, order=3)
    assert np.array_equal(tomo.affine_cubic(vol, tf, off), ref)


def load_case(name):
    f = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return f, json.loads(str(f["meta"]))


def preprocessed(name, device="cpu"):
    from py4dstem_gb300 import DataCube, PtychographicTomography

    f, meta = load_case(name)
    dcs = [DataCube(f["datacube"][i].astype(np.float32), r_pixel_size=meta["r_pixel_size"][i],
                    r_pixel_units="A", q_pixel_size=meta["q_pixel_size"][i],
                    q_pixel_units="mrad") for i in range(len(meta["seeds"]))]
    extra = {}
    if "initial_object_guess" in f.files:
        extra["initial_object_guess"] = f["initial_object_guess"].copy()
    p = PtychographicTomography(tilt_orientation_matrices=list(f["tilt_matrices"]),
                                datacube=dcs, initial_scan_positions=list(f["scan_positions_ang"]),
                                verbose=False, device=device, **meta["ctor"], **extra)
    p.preprocess(**meta["preprocess"])
    return p, f, meta


@pytest.mark.parametrize("name", TOMO_CASES)
def test_host_preprocess_matches_reference(name):
    p, f, _ = preprocessed(name)
    assert np.array_equal(np.asarray(p._mean_diffraction_intensity, np.float32),
                          f["pre_mean_intensity"])
    assert np.array_equal(p._positions_px_all, f["pre_positions_px"])
    assert np.array_equal(np.stack(p._probes_all), f["pre_probe_initial"])
    assert np.array_equal(p._object, f["pre_object_initial"])
    assert np.array_equal(p._amplitudes.astype(np.float64).sum(axis=(-2, -1)),
                          f["pre_amplitude_sums"])
    assert np.array_equal(p._propagator_arrays, f["pre_propagators"])


def oracle_for(p, f, meta):
    return tomo.TomographyOracle(
        volume=f["pre_object_initial"], probes=f["pre_probe_initial"], amplitudes=p._amplitudes,
        positions_px=f["pre_positions_px"], cum_counts=p._cum_probes_per_measurement,
        mean_intensity=f["pre_mean_intensity"], tilt_matrices=f["tilt_matrices"],
        num_slices=meta["ctor"]["num_slices"], propagators=f["pre_propagators"])


@pytest.mark.parametrize("name", TOMO_CASES)
def test_oracle_matches_reference(name):
    """Equal up to the last bits of the float64 rotation of the update: the
    sequential case (no rotation of the update) agrees in every error value."""
    p, f, meta = preprocessed(name)
    o = oracle_for(p, f, meta).reconstruct(sampling=tuple(p.sampling), **meta["reconstruct"])
    err = np.asarray(o.error_iterations)
    ref_err = f["out_error_iterations"]
    assert np.abs(err - ref_err).max() <= 1e-7 * np.abs(ref_err).max()
    scale = np.abs(f["out_object"]).max()
    assert np.abs(o.volume - f["out_object"]).max() <= 1e-6 * scale
    pr = np.stack(o.probes)
    assert np.abs(pr - f["out_probes_corner"]).max() <= 1e-6 * np.abs(pr).max()
    if name == "tomo_gd_sequential":
        assert np.array_equal(err, ref_err)


def test_unsupported_options_raise_before_gpu():
    p, _, _ = preprocessed("tomo_gd_sequential")
    for kw in (dict(reconstruction_method="RAAR"), dict(fix_positions=False),
               dict(q_lowpass=0.5), dict(tv_denoise_weights=[0.1, 0.1])):
        with pytest.raises(NotImplementedError):
            p.reconstruct(num_iter=1, device="gpu", progress_bar=False, **kw)
    with pytest.raises(NotImplementedError):
        p._return_self_consistency_errors()


def test_constructor_checks():
    from py4dstem_gb300 import PtychographicTomography

    with pytest.raises(NotImplementedError):
        PtychographicTomography(energy=300e3, num_slices=2,
                                tilt_orientation_matrices=[np.eye(3)], object_type="complex")
    with pytest.raises(ValueError):
        PtychographicTomography(energy=300e3, num_slices=2,
                                tilt_orientation_matrices=[np.eye(3)], not_a_parameter=1.0)


def test_reset_semantics():
    """MultipleMeasurementsMethodsMixin._reset_reconstruction
    (ptychographic_methods.py:3409-3462): reset=True restores the initial
    volume, probes and positions; reset=None after a run warns and continues."""
    p, _, _ = preprocessed("tomo_gd_sequential")
    vol0 = p._object.copy()
    probes0 = [pr.copy() for pr in p._probes_all]
    pos0 = p._positions_px_all.copy()
    p._object += 1.0
    p._probes_all = [pr * 2 for pr in p._probes_all]
    p._positions_px_all += 0.5
    p.error = 0.1
    p.error_iterations = [0.2, 0.1]
    with pytest.warns(UserWarning, match="Continuing"):
        p._reset_tomography(store_iterations=False, reset=None)
    assert p.error_iterations == [0.2, 0.1]
    p._reset_tomography(store_iterations=True, reset=True)
    assert p.error_iterations == [] and p.object_iterations == [] and p.probe_iterations == []
    np.testing.assert_array_equal(p._object, vol0)
    np.testing.assert_array_equal(p._positions_px_all, pos0)
    for a, b in zip(p._probes_all, probes0):
        np.testing.assert_array_equal(a, b)
    # the initial arrays are copies: changing the state leaves them alone
    p._object += 1.0
    np.testing.assert_array_equal(p._object_initial, vol0)


def test_host_preprocess_mask_and_shifts_match_reference():
    """One 2D positions mask for every tilt (tiled, with the reference's
    warning) and forced centre-of-mass shifts for the first tilt only."""
    from py4dstem_gb300 import DataCube, PtychographicTomography

    f, meta = load_case("tomo_pre_mask_shifts")
    mask = f["positions_mask"]
    dcs = [DataCube(f["datacube"][i].astype(np.float32), r_pixel_size=meta["r_pixel_size"][i],
                    r_pixel_units="A", q_pixel_size=meta["q_pixel_size"][i],
                    q_pixel_units="mrad") for i in range(len(meta["seeds"]))]
    p = PtychographicTomography(
        tilt_orientation_matrices=list(f["tilt_matrices"]), datacube=dcs,
        initial_scan_positions=[pos[mask.ravel()] for pos in f["scan_positions_ang"]],
        positions_mask=mask, verbose=False, device="cpu", **meta["ctor"])
    with pytest.warns(UserWarning, match="assumed the same for all measurements"):
        p.preprocess(**meta["preprocess"])
    np.testing.assert_array_equal(p._cum_probes_per_measurement, f["pre_cum_counts"])
    assert np.array_equal(np.asarray(p._mean_diffraction_intensity, np.float32),
                          f["pre_mean_intensity"])
    assert np.array_equal(p._positions_px_all, f["pre_positions_px"])
    assert np.array_equal(np.stack(p._probes_all), f["pre_probe_initial"])
    assert np.array_equal(p._object, f["pre_object_initial"])
    assert np.array_equal(p._amplitudes.astype(np.float64).sum(axis=(-2, -1)),
                          f["pre_amplitude_sums"])
    assert np.array_equal(p._propagator_arrays, f["pre_propagators"])
