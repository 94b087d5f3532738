"""The host-side global affine constraint of corrected positions
(py4dstem_gb300.positions) against the oracle's restatement, which is pinned on
the reference fixture ss_gd_poscorr_affine: same positions and the same draws
from NumPy's global generator."""

import numpy as np

from oracle.ptycho_np import Oracle
from py4dstem_gb300.positions import AffineTransform, affine_constraint, fit_affine


def _positions(seed, J=144):
    rng = np.random.default_rng(seed)
    g = np.arange(12) * 2.0
    xx, yy = np.meshgrid(g, g, indexing="ij")
    x0 = (np.stack([xx.ravel(), yy.ravel()], -1)[:J] + 40).astype(np.float32)
    A = np.array([[1.02, 0.03], [-0.01, 0.97]], np.float32)
    x1 = ((x0 - x0.mean(0)) @ A + x0.mean(0) + np.float32(0.4)).astype(np.float32)
    x1 += rng.normal(0, 0.05, x1.shape).astype(np.float32)
    x1[:5] += 40.0  # outliers beyond the 16 px inlier distance
    return x0, x1


def test_affine_constraint_matches_oracle():
    x0, x1 = _positions(3)

    np.random.seed(11)
    new, tf = affine_constraint(x0, x1)
    after = np.random.random()
    stub = Oracle.__new__(Oracle)  # only the two position arrays are used
    stub.positions_initial = x0
    stub.positions_px = x1.copy()
    np.random.seed(11)
    stub.positions_affine_constraint()
    assert np.random.random() == after  # the same number of draws
    np.testing.assert_array_equal(new, stub.positions_px)
    assert new.dtype == np.float32
    # the outliers do not drag the fit (the decomposition keeps |angle| only,
    # as the reference's does, so a small rotation of either sign fits to it)
    assert np.abs(new[5:] - x1[5:]).max() < 2.0


def test_exact_affine_fit_and_identity():
    x0, _ = _positions(4)
    tf0 = AffineTransform(scale0=1.1, scale1=0.9, shear1=0.05, angle=0.1,
                          t0=np.float32(1.5), t1=np.float32(-2.0))
    com = x0.mean(0)
    x1 = tf0(x0, origin=com).astype(np.float32)
    tf, err = fit_affine(x0, x1, origin=com)
    assert err < 1e-3
    np.testing.assert_allclose(tf.matrix(), tf0.matrix(), atol=1e-5)
    # a degenerate system falls back to the identity
    same = np.repeat(x0[:1], 10, axis=0)
    tf, _ = fit_affine(same, same, origin=same.mean(0))
    assert tf == AffineTransform()
