"""Pin the oracle and the host preprocessing against the reference's own outputs.

The golden fixtures hold what the unmodified py4DSTEM 0.14.18 CPU path returned
(tests/golden/make_golden.py). Here, on the CPU:
  * py4dstem_gb300's host preprocess must reproduce the reference's preprocessed
    state bit for bit;
  * oracle/ptycho_np.py (float32) run on that state must reproduce the reference's
    reconstruction bit for bit (same NumPy operations, same order).
"""

import numpy as np
import pytest

from golden_io import Golden, PrepGolden, names, prep_names
from oracle.ptycho_np import Oracle


@pytest.mark.parametrize("name", names())
def test_preprocess_matches_reference(name):
    g = Golden(name)
    p = g.build(device="cpu")  # device="cpu": the host preprocess, no GPU
    assert np.float32(p._mean_diffraction_intensity) == g.pre["mean_intensity"]
    np.testing.assert_array_equal(p._positions_px, g.pre["positions_px"])
    np.testing.assert_array_equal(p._probe, g.pre["probe_initial"])
    np.testing.assert_array_equal(p._object, g.pre["object_initial"])
    np.testing.assert_array_equal(p._object_fov_mask, g.pre["fov_mask"])
    np.testing.assert_array_equal(p._amplitudes.astype(np.float64).sum(axis=(-2, -1)),
                                  g.pre["amplitude_sums"])
    np.testing.assert_array_equal(p._amplitudes[0], g.pre["amplitude_first"])
    np.testing.assert_array_equal(p._amplitudes[-1], g.pre["amplitude_last"])


@pytest.mark.parametrize("name", prep_names())
def test_preprocess_options_match_reference(name):
    """Rotation search (curl and divergence, custom angles, forced transpose),
    detector and positions masks, corner crop, per-pattern centre of mass and the
    surface fits: the host preprocess gives the reference's bits."""
    g = PrepGolden(name)
    g.check(g.build(device="cpu"))


@pytest.mark.parametrize("name", names())
def test_oracle_reproduces_reference(name):
    g = Golden(name)
    p = g.build(device="cpu")
    o = Oracle(g.state(p)).reconstruct(**g.oracle_kwargs())
    np.testing.assert_array_equal(np.asarray(o.error_iterations, dtype=np.float64),
                                  g.out["error_iterations"])
    np.testing.assert_array_equal(o.object, g.out["object"])
    np.testing.assert_array_equal(o.probe, g.out["probe_corner"])
    np.testing.assert_array_equal(o.positions_px, g.out["positions_px"])
    np.testing.assert_array_equal(
        o.self_consistency_errors(g.meta["reconstruct"].get("max_batch_size")),
        g.out["self_consistency_errors"])


def test_oracle_float64_close_to_float32():
    """The FP64 evaluation of the same model stays within the float32 noise floor."""
    g = Golden("ms_gd_T3")
    p = g.build(device="cpu")
    o32 = Oracle(g.state(p)).reconstruct(**g.oracle_kwargs())
    o64 = Oracle(g.state(p), "float64").reconstruct(**g.oracle_kwargs())
    e32 = np.asarray(o32.error_iterations)
    e64 = np.asarray(o64.error_iterations)
    assert np.max(np.abs(e32 - e64) / e64) < 1e-3
