"""PtychographicTomography on the GPU.

* Volume kernels against the reference's own outputs
  (tests/golden/tomo_volume_ops.npz: _rotate_zxy_volume on float32 and float64
  volumes, _project_sliced_object, _expand_sliced_object), against SciPy on
  edge shapes, and the float32 updates against NumPy.
* Whole reconstructions (collective and sequential updates from a smooth
  initial volume; the default zero start against the float32 floor) against
  the reference's result (tests/golden/tomo_*.npz).
* The device preprocess against the host one on the same machine.
"""

import os

import numpy as np
import pytest

from test_tomography_oracle import GOLDEN, TOMO_CASES, preprocessed

pytestmark = pytest.mark.gpu


def _ops(torch, shape, num_slices=1):
    from py4dstem_gb300.tomography import VolumeOps

    return VolumeOps(shape, num_slices, torch.device("cuda"))


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_rotation_kernel_matches_reference(cuda):
    torch = cuda
    z = np.load(os.path.join(GOLDEN, "tomo_volume_ops.npz"))
    vol, vol64 = z["volume"], z["volume64"]
    ops = _ops(torch, vol.shape)
    src32, src64 = _dev(torch, vol), _dev(torch, vol64)
    for k in range(4):
        m = z[f"matrix_{k}"]
        ref32, ref64 = z[f"rot32_{k}"], z[f"rot64_{k}"]
        out = torch.empty_like(src32)
        ops.rotate(src32, out, m, 0)
        got = out.cpu().numpy()
        # float64 arithmetic as SciPy's; the last float64 bits may round a
        # float32 voxel the other way
        assert np.mean(got == ref32) > 0.999
        assert np.abs(got - ref32).max() <= 1e-6 * np.abs(ref32).max()
        out64 = torch.empty_like(src64)
        ops.rotate(src64, out64, m, 1)
        assert np.abs(out64.cpu().numpy() - ref64).max() < 1e-13
        # add into a float32 volume (the collective update)
        base = np.linspace(-1, 1, vol.size, dtype=np.float32).reshape(vol.shape)
        acc = _dev(torch, base)
        ops.rotate(src64, acc, m, 2)
        want = (base.astype(np.float64) + ref64).astype(np.float32)
        assert np.mean(acc.cpu().numpy() == want) > 0.999
        assert np.abs(acc.cpu().numpy() - want).max() <= 1e-6
        # in place (output over the input)
        inplace = src32.clone()
        ops.rotate(inplace, inplace, m, 0)
        assert torch.equal(inplace, out)


@pytest.mark.parametrize("shape", [(1, 5, 7), (2, 3, 4), (5, 1, 6), (6, 6, 2)])
def test_rotation_kernel_edge_shapes(cuda, shape):
    from scipy.ndimage import affine_transform

    from py4dstem_gb300.tomography import rotation_transform

    torch = cuda
    rng = np.random.default_rng(sum(shape))
    vol = rng.random(shape).astype(np.float32)
    t = np.deg2rad(23.0)
    rot = np.array([[1, 0, 0], [0, np.cos(t), -np.sin(t)], [0, np.sin(t), np.cos(t)]])
    tf, off = rotation_transform(shape, rot)
    ref = affine_transform(vol, tf, offset=off, order=3)
    ops = _ops(torch, shape)
    src = _dev(torch, vol)
    out = torch.empty_like(src)
    ops.rotate(src, out, rot, 0)
    got = out.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-6 * max(1.0, np.abs(ref).max())


def test_project_expand_and_updates_bit_exact(cuda):
    torch = cuda
    z = np.load(os.path.join(GOLDEN, "tomo_volume_ops.npz"))
    vol = z["volume"]
    n0 = vol.shape[0]
    src = _dev(torch, vol)
    rng = np.random.default_rng(3)
    for t in (1, 3, 6, 7):
        ops = _ops(torch, vol.shape, t)
        sliced = torch.empty((t,) + vol.shape[1:], dtype=torch.float32, device="cuda")
        ops.project(src, sliced)
        assert np.array_equal(sliced.cpu().numpy(), z[f"project_{t}"])
        upd = _dev(torch, z[f"update_{t}"])
        zero = torch.zeros_like(upd)
        out64 = torch.empty(vol.shape, dtype=torch.float64, device="cuda")
        ops.expand(upd, zero, out64, 1)
        assert np.array_equal(out64.cpu().numpy(), z[f"expand_{t}"])
        # (new - old) expanded and added into a float32 volume
        new = z[f"update_{t}"] + rng.normal(size=z[f"update_{t}"].shape).astype(np.float32)
        old = z[f"update_{t}"]
        acc = src.clone()
        ops.expand(_dev(torch, new), _dev(torch, old), acc, 2)
        from oracle.tomography_np import expand_sliced

        want = (vol.astype(np.float64) + expand_sliced(new - old, n0)).astype(np.float32)
        assert np.array_equal(acc.cpu().numpy(), want)
    ops = _ops(torch, vol.shape)
    coll = rng.normal(size=vol.shape).astype(np.float32)
    acc = src.clone()
    ops.add_scaled(acc, _dev(torch, coll), 3)
    assert np.array_equal(acc.cpu().numpy(), vol + coll / 3)
    signed = (vol - np.float32(0.5)).astype(np.float32)
    acc = _dev(torch, signed)
    ops.constraints(acc, 1e-3, True)
    want = signed.copy()
    want -= 1e-3
    assert np.array_equal(acc.cpu().numpy(), want.clip(0.0))


def _distances(p_object, p_probes, p_errors, f):
    ref_err = f["out_error_iterations"]
    d_err = np.abs(np.asarray(p_errors) - ref_err).max() / np.abs(ref_err).max()
    d_obj = np.abs(p_object - f["out_object"]).max() / np.abs(f["out_object"]).max()
    d_pr = (np.abs(np.stack(p_probes) - f["out_probes_corner"]).max()
            / np.abs(f["out_probes_corner"]).max())
    return np.array([d_err, d_obj, d_pr])


@pytest.mark.parametrize("name", ["tomo_gd_collective", "tomo_gd_sequential",
                                  "tomo_gd_gaussian"])
def test_reconstruction_matches_reference(cuda, name):
    """From a smooth initial volume (well conditioned: a change of the float32
    FFT alone moves the reference's result by about 3e-7) the float32 kernels
    agree with the reference, whose amplitudes and Fourier projection are
    float64, to 5e-6 in the errors and 1e-5 in the volume and probes (relative
    to their largest values; measured on a GB300: 2e-7, 6e-7, 7e-7)."""
    p, f, meta = preprocessed(name)
    p.reconstruct(progress_bar=False, device="gpu", **meta["reconstruct"])
    assert p.object.shape == f["out_object"].shape and p.object.dtype == np.float32
    assert len(p.probe) == len(meta["seeds"])
    d = _distances(p.object, p._probes_all, p.error_iterations, f)
    print(f"{name}: error {d[0]:.2e} volume {d[1]:.2e} probes {d[2]:.2e}")
    assert d[0] < 5e-6 and d[1] < 1e-5 and d[2] < 1e-5, d


def test_zero_start_within_float32_floor(cuda):
    """From the default zero volume the first steps are ill-conditioned: the
    same model under a more accurate float32 FFT (every FFT in complex128,
    rounded) already moves the reference's result by about 1e-2. The GPU result
    must lie within 3x that distance (errors, volume, probes)."""
    from test_tomography_oracle import oracle_for

    name = "tomo_gd_zero_start"
    p, f, meta = preprocessed(name)
    o = oracle_for(p, f, meta)
    o.fft_round_trip = True
    o.reconstruct(**meta["reconstruct"])
    floor = _distances(o.volume, o.probes, o.error_iterations, f)
    p.reconstruct(progress_bar=False, device="gpu", **meta["reconstruct"])
    d = _distances(p.object, p._probes_all, p.error_iterations, f)
    print(f"{name}: gpu {d} floor {floor}")
    assert np.all(d <= 3 * floor + 1e-7), (d, floor)


def test_device_preprocess_matches_host(cuda):
    name = TOMO_CASES[0]
    host, _, _ = preprocessed(name, device="cpu")
    dev, _, _ = preprocessed(name, device="gpu")
    assert np.array_equal(np.asarray(dev._mean_diffraction_intensity),
                          np.asarray(host._mean_diffraction_intensity))
    assert np.array_equal(dev._amplitudes, host._amplitudes)
    assert np.array_equal(dev._positions_px_all, host._positions_px_all)
    assert np.array_equal(dev._object, host._object)
