"""Device preprocessing (device="gpu") against the reference and the host path.

The centre of mass, the rotation search and the normalised amplitudes must
carry the reference's float32 bits (the kernels follow NumPy's summation order
and roundings); the probe-overlap map goes through float32 FFTs and must agree
to rounding, with the same field-of-view mask.
"""

import numpy as np
import pytest

from golden_io import Golden, PrepGolden, names, prep_names, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", prep_names())
def test_device_preprocess_options_match_host_and_reference(cuda, name):
    """The device preprocess gives the host path's bits on the same machine, and
    the reference's (computed on x86) wherever no host FFT precedes the centre of
    mass: Fourier resampling and the initial probe are NumPy FFTs on the host,
    whose float32 bits differ between CPU architectures."""
    g = PrepGolden(name)
    d = g.build(device="gpu")
    PrepGolden.same_state(d, g.build(device="cpu"))
    if g.meta["preprocess"].get("reshaping_method") != "fourier":
        g.check(d, probe_exact=False)


@pytest.mark.parametrize("name", names())
def test_device_preprocess_matches_reference(cuda, name):
    g = Golden(name)
    p = g.build(device="gpu")
    assert np.float32(p._mean_diffraction_intensity) == g.pre["mean_intensity"]
    np.testing.assert_array_equal(p._positions_px, g.pre["positions_px"])
    # the probe is host NumPy work (see PrepGolden.check)
    assert rel_l2(p._probe, g.pre["probe_initial"]) < 1e-6
    np.testing.assert_array_equal(p._object_fov_mask, g.pre["fov_mask"])
    np.testing.assert_array_equal(p._amplitudes.astype(np.float64).sum(axis=(-2, -1)),
                                  g.pre["amplitude_sums"])
    np.testing.assert_array_equal(p._amplitudes[0], g.pre["amplitude_first"])
    np.testing.assert_array_equal(p._amplitudes[-1], g.pre["amplitude_last"])


def _host():
    from py4dstem_gb300 import SingleslicePtychography

    return SingleslicePtychography(energy=300e3, device="cpu", verbose=False)


@pytest.mark.parametrize("shape,masked", [((5, 7, 48, 48), False), ((3, 4, 96, 96), True),
                                          ((2, 3, 128, 128), False), ((4, 4, 37, 41), True),
                                          ((1, 2, 5, 3), False), ((2, 2, 256, 256), True)])
def test_pattern_com_bits(cuda, shape, masked):
    from py4dstem_gb300 import device_preprocess

    rng = np.random.default_rng(sum(shape))
    data = rng.poisson(20.0, size=shape).astype(np.float32) * rng.random(shape, dtype=np.float32)
    mask = rng.random(shape[-2:]) > 0.2 if masked else None
    kx = np.arange(shape[-2], dtype=np.float32)
    ky = np.arange(shape[-1], dtype=np.float32)
    kya, kxa = np.meshgrid(ky, kx)
    im = data * mask if masked else data
    isum = np.sum(im, axis=(-2, -1))
    ref_x = np.sum(im * kxa[None, None], axis=(-2, -1)) / isum
    ref_y = np.sum(im * kya[None, None], axis=(-2, -1)) / isum
    cx, cy = device_preprocess.pattern_com(device_preprocess.upload_intensities(data), mask)
    np.testing.assert_array_equal(cx.reshape(shape[:2]), ref_x)
    np.testing.assert_array_equal(cy.reshape(shape[:2]), ref_y)


@pytest.mark.parametrize("shape", [(4, 5, 64, 64), (3, 3, 37, 41)])
@pytest.mark.parametrize("vectorized", [True, False])
def test_pattern_com_float64_mask_bits(cuda, shape, vectorized):
    """A float64 mask (e.g. a Fourier-resampled one): float64 sums in the
    vectorised form, the in-place float32 product in the per-pattern loop."""
    from py4dstem_gb300 import device_preprocess

    rng = np.random.default_rng(sum(shape) + 7)
    data = rng.poisson(20.0, size=shape).astype(np.float32)
    mask = rng.random(shape[-2:]) * 1.3
    kx = np.arange(shape[-2], dtype=np.float32)
    ky = np.arange(shape[-1], dtype=np.float32)
    kya, kxa = np.meshgrid(ky, kx)
    if vectorized:
        im = data * mask
        isum = np.sum(im, axis=(-2, -1))
        ref_x = np.sum(im * kxa[None, None], axis=(-2, -1)) / isum
        ref_y = np.sum(im * kya[None, None], axis=(-2, -1)) / isum
        assert ref_x.dtype == np.float64
    else:
        ref_x = np.zeros(shape[:2], np.float32)
        ref_y = np.zeros(shape[:2], np.float32)
        for rx in range(shape[0]):
            for ry in range(shape[1]):
                mi = np.array(data[rx, ry])
                mi *= mask
                t = mi.sum()
                ref_x[rx, ry] = np.sum(mi * kxa) / t
                ref_y[rx, ry] = np.sum(mi * kya) / t
    cx, cy = device_preprocess.pattern_com(device_preprocess.upload_intensities(data), mask,
                                           vectorized)
    assert cx.dtype == ref_x.dtype
    np.testing.assert_array_equal(cx.reshape(shape[:2]), ref_x)
    np.testing.assert_array_equal(cy.reshape(shape[:2]), ref_y)


@pytest.mark.parametrize("scan", [(3, 3), (13, 17), (64, 64), (130, 97)])
@pytest.mark.parametrize("divergence", [False, True])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_rotation_search_bits(cuda, scan, divergence, dtype):
    from py4dstem_gb300 import device_preprocess

    rng = np.random.default_rng(scan[0] * 1000 + scan[1])
    cnx = rng.normal(size=scan).astype(dtype) * 0.01
    cny = rng.normal(size=scan).astype(dtype) * 0.01
    deg = np.arange(-89.0, 90.0, 1.0).astype(np.float32)
    rad = np.deg2rad(deg)[:, None, None]
    host = _host()
    ref = [host._curl_or_div(*host._rotated(cnx[None], cny[None], rad, t), divergence,
                             axis=(-2, -1)) for t in (False, True)]
    vals = device_preprocess.rotation_values(cnx, cny, np.cos(rad), np.sin(rad), divergence)
    np.testing.assert_array_equal(vals[0], ref[0])
    np.testing.assert_array_equal(vals[1], ref[1])


@pytest.mark.parametrize("qshape,crop,pmask", [((64, 64), False, False), ((96, 96), True, True),
                                               ((128, 128), False, True), ((40, 52), True, False),
                                               ((256, 256), False, True), ((256, 256), True, False)])
def test_normalize_bits(cuda, qshape, crop, pmask):
    from py4dstem_gb300 import device_preprocess

    rng = np.random.default_rng(qshape[0] + qshape[1])
    rs = (6, 5)
    data = (rng.poisson(30.0, size=rs + qshape) - 2.0).astype(np.float32)  # some negatives
    cfx = (qshape[0] / 2 + rng.normal(size=rs) * 3).astype(np.float32)
    cfy = (qshape[1] / 2 + rng.normal(size=rs) * 3).astype(np.float32)
    mask = rng.random(rs) > 0.25 if pmask else None
    host = _host()
    ref, ref_mean, ref_crop, ref_shape = host._normalize_intensities(data, cfx, cfy, mask, crop,
                                                                     False)
    dev = device_preprocess.upload_intensities(data)
    gpu = _host()
    gpu._device = "gpu"
    amps, mean, crop_mask, crop_shape = gpu._normalize_intensities_device(dev, cfx, cfy, mask,
                                                                          crop)
    np.testing.assert_array_equal(amps.cpu().numpy(), ref)
    assert np.float32(mean) == np.float32(ref_mean)
    assert tuple(crop_shape) == tuple(ref_shape)
    if crop:
        np.testing.assert_array_equal(crop_mask, ref_crop)


@pytest.mark.parametrize("roi,J,batch", [(64, 300, 64), (128, 100, None), (48, 77, 1000),
                                         (256, 40, 16)])
def test_probe_overlap_close(cuda, roi, J, batch):
    from py4dstem_gb300 import device_preprocess
    from py4dstem_gb300.optics import ComplexProbe

    rng = np.random.default_rng(roi + J)
    host = _host()
    host._region_of_interest_shape = np.array((roi, roi))
    host._object_shape = (roi + 64, roi + 80)
    host._num_diffraction_patterns = J
    host._positions_px = (rng.random((J, 2)) * np.array(host._object_shape)).astype(np.float32)
    probe = ComplexProbe(gpts=(roi, roi), sampling=(0.25, 0.25), energy=300e3,
                         semiangle_cutoff=20.0, parameters={"C10": -100.0}).build()._array
    ref = host._probe_overlap(probe, batch)
    got = device_preprocess.probe_overlap(probe, host._positions_px, host._object_shape, batch)
    assert got.shape == ref.shape and got.dtype == np.float32
    assert np.max(np.abs(got - ref)) <= 1e-5 * np.max(ref)


def test_storage_cpu_gets_page_locked_amplitudes(cuda):
    from py4dstem_gb300 import engine

    g = Golden("ss_gd_det128")
    p = g.build(device="gpu", storage="cpu")
    assert engine.mapped_host_address(p._amplitudes) is not None
    np.testing.assert_array_equal(p._amplitudes[0], g.pre["amplitude_first"])
