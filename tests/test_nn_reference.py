"""The NumPy reference of the learned initializer's network checked on the CPU:
its convolution gradients against central finite differences, and its pooling
and upsampling adjoints against their forward maps."""

import numpy as np

import nn_reference as ref


def test_conv_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((1, 5, 8, 3))
    w = rng.standard_normal((4, 9, 3))
    dy = rng.standard_normal((1, 5, 8, 4))

    def loss(xv, wv):
        return float(np.sum(ref.conv3x3(xv, wv) * dy))

    dx = ref.conv3x3_backward_data(dy, w)
    dw, db = ref.conv3x3_backward_weight(x, dy)
    eps = 1e-6
    for idx in [(0, 0, 0, 0), (0, 4, 7, 2), (0, 2, 3, 1), (0, 0, 7, 0)]:
        xp, xm = x.copy(), x.copy()
        xp[idx] += eps
        xm[idx] -= eps
        assert abs((loss(xp, w) - loss(xm, w)) / (2 * eps) - dx[idx]) < 1e-6
    for idx in [(0, 0, 0), (3, 8, 2), (1, 4, 1)]:
        wp, wm = w.copy(), w.copy()
        wp[idx] += eps
        wm[idx] -= eps
        assert abs((loss(x, wp) - loss(x, wm)) / (2 * eps) - dw[idx]) < 1e-6
    np.testing.assert_allclose(db, dy.sum(axis=(0, 1, 2)))


def test_pool_and_upsample_adjoints():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2, 4, 6, 3))
    p, idx = ref.maxpool(x)
    d = rng.standard_normal(p.shape)
    g = ref.maxpool_backward(d, idx, x.shape)
    # gradient of sum(maxpool(x) * d): d at the argmax of each window
    assert np.isclose(np.sum(g * x), np.sum(p * d))
    u = rng.standard_normal((1, 3, 2, 2))
    v = rng.standard_normal((1, 6, 4, 2))
    assert np.isclose(np.sum(ref.upsample(u) * v), np.sum(u * ref.upsample_backward(v)))


def test_bf16_rounding_is_nearest_even():
    a = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-40], np.float32)
    r = ref.bf16_round(a)
    assert r[0] == 1.0 and r[1] == 1.0  # halfway: to even
    assert r[2] == np.float32(1.0078125)
    assert r[3] == -2.5
