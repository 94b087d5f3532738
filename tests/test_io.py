"""Saving and reading a reconstruction (the reference's to_h5 / read content in
an .npz file), on the host."""

import numpy as np
import pytest

import py4dstem_gb300 as pg
from golden_io import Golden


@pytest.mark.parametrize("name", ["ss_gd_potential", "ms_gd_T3", "mixed_gd_M3", "mms_gd_T3M2"])
def test_save_read_round_trip(tmp_path, name):
    g = Golden(name)
    p = g.build(device="cpu")
    # a reconstruction state as reconstruct() leaves it
    p._object = (np.asarray(p._object) * np.float32(1.01)).astype(np.asarray(p._object).dtype)
    p._probe = (np.asarray(p._probe) * np.complex64(0.99 + 0.01j)).astype(np.complex64)
    p.error_iterations = [0.5, 0.25, 0.125]
    p.object_iterations = [np.asarray(p._object)] * 3
    p.probe_iterations = [p.probe_centered] * 3
    p.set_save_defaults(save_datacube=True, save_iterations_frequency=2)
    path = tmp_path / f"{name}.npz"
    p.save(path)

    q = pg.read(path, device="cpu")
    assert type(q) is type(p)
    np.testing.assert_array_equal(q._object, p._object)
    np.testing.assert_array_equal(q._probe, p._probe)
    np.testing.assert_array_equal(q.object, p._object)
    np.testing.assert_array_equal(q._positions_px, p._positions_px)
    assert q.error_iterations == p.error_iterations and q.error == 0.125
    assert len(q.object_iterations) == 2  # iterations 0 and 2
    assert q._rotation_best_rad == p._rotation_best_rad
    assert q._rotation_best_transpose == p._rotation_best_transpose
    assert q._num_diffraction_patterns == p._num_diffraction_patterns
    assert tuple(q._region_of_interest_shape) == tuple(p._region_of_interest_shape)
    assert q.sampling == pytest.approx(p.sampling)
    assert q._polar_parameters == p._polar_parameters
    for key in ("_num_slices", "_num_probes"):
        assert getattr(q, key) == getattr(p, key)
    np.testing.assert_array_equal(np.asarray(getattr(q, "_slice_thicknesses", 0)),
                                  np.asarray(getattr(p, "_slice_thicknesses", 0)))
    np.testing.assert_allclose(q.positions, p.positions, rtol=0, atol=1e-4)

    # continuing: preprocess again from the saved datacube, with the saved object
    # and probe as the initial guesses
    q.preprocess(**g.meta["preprocess"])
    np.testing.assert_array_equal(q._object, p._object)
    np.testing.assert_array_equal(q._probe, p._probe)
    np.testing.assert_allclose(q._positions_px, p._positions_px, rtol=0, atol=1e-3)
    np.testing.assert_array_equal(q._amplitudes, p._amplitudes)


def test_save_requires_preprocess(tmp_path):
    p = pg.SingleslicePtychography(energy=300e3, device="cpu")
    with pytest.raises(ValueError):
        p.save(tmp_path / "x.npz")


def test_read_without_preprocess_asks_for_it(tmp_path):
    g = Golden("ss_gd_potential")
    p = g.build(device="cpu")
    p.save(tmp_path / "r.npz")
    q = pg.read(tmp_path / "r.npz", device="cpu")
    with pytest.raises(ValueError, match="GPU only"):
        q.reconstruct(num_iter=1)


def test_tomography_save_read_round_trip(tmp_path):
    from test_tomography_oracle import preprocessed

    p, _, meta = preprocessed("tomo_gd_sequential")
    # a reconstruction state as reconstruct() leaves it
    p._object = (p._object * np.float32(1.01) + np.float32(1e-3)).astype(np.float32)
    p._probes_all = [(pr * np.complex64(0.99 + 0.01j)).astype(np.complex64)
                     for pr in p._probes_all]
    p.error_iterations = [0.5, 0.25, 0.125]
    p.object_iterations = [p._object] * 3
    p.probe_iterations = [p.probe_centered] * 3
    p.set_save_defaults(save_datacube=True, save_iterations_frequency=2)
    path = tmp_path / "tomo.npz"
    p.save(path)

    q = pg.read(path, device="cpu")
    assert type(q) is type(p)
    np.testing.assert_array_equal(q._object, p._object)
    np.testing.assert_array_equal(q.object, p._object)
    assert len(q._probes_all) == len(p._probes_all)
    for a, b in zip(q._probes_all, p._probes_all):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(q._positions_px_all, p._positions_px_all)
    np.testing.assert_array_equal(q._cum_probes_per_measurement, p._cum_probes_per_measurement)
    np.testing.assert_array_equal(np.asarray(q._mean_diffraction_intensity),
                                  np.asarray(p._mean_diffraction_intensity))
    np.testing.assert_array_equal(q._propagator_arrays, p._propagator_arrays)
    for a, b in zip(q._tilt_orientation_matrices, p._tilt_orientation_matrices):
        np.testing.assert_array_equal(a, b)
    assert q.error_iterations == p.error_iterations and q.error == 0.125
    assert len(q.object_iterations) == 2 and len(q.probe_iterations[0]) == len(p._probes_all)
    assert q.sampling == pytest.approx(p.sampling)
    assert q._num_slices == p._num_slices and q._num_measurements == p._num_measurements
    # the saved datacubes come back: preprocess() again from the saved state
    q.preprocess(**meta["preprocess"])
    np.testing.assert_array_equal(q._amplitudes, p._amplitudes)
    np.testing.assert_array_equal(q._object, p._object)  # the saved volume as the guess
    for a, b in zip(q._probes_all, p._probes_all):
        np.testing.assert_array_equal(a, b)
