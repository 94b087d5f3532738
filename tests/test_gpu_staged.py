"""The staged batch-wide kernels against the oracle: the 256 x 256 region of
interest (gradient descent of every model with each option, the constraints
over several iterations, the forward-only errors, the probe aperture
constraint and the object gradient) and far fields resampled to a detector of
another shape at the fused sizes. Tolerances as for the fused kernels (the
256-point transforms round like the 128-point ones: two radix-16 passes).
The reference-run fixtures with region_of_interest_shape (ss_gd_resample_*,
mixed_gd_resample, ms_gd_resample) go through tests/test_gpu_golden.py."""

import ctypes

import numpy as np
import pytest

from gpu_helpers import gpu_reconstruct, make_state, rel
from oracle.ptycho_np import Oracle

pytestmark = pytest.mark.gpu

OFF = dict(fix_probe_com=False, fix_potential_baseline=False, orthogonalize_probe=False)


def compare(state, tol_obj, tol_probe, tol_err, **kw):
    o = Oracle(state).reconstruct(**kw)
    g_obj, g_probe, g_err = gpu_reconstruct(state, **kw)
    d_obj = rel(g_obj, o.object)
    d_probe = rel(g_probe, o.probe)
    d_err = float(np.max(np.abs(np.array(g_err) - np.array(o.error_iterations))
                         / np.abs(np.array(o.error_iterations))))
    print(f"obj {d_obj:.2e} probe {d_probe:.2e} err {d_err:.2e}")
    assert d_obj < tol_obj, d_obj
    assert d_probe < tol_probe, d_probe
    assert d_err < tol_err, d_err


def test_gradient_descent_256(cuda):
    st = make_state(S=256, J=16, seed=256)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=8, seed_random=1, **OFF)


@pytest.mark.parametrize("potential,masked,fix_probe", [(True, False, False),
                                                        (False, True, True)])
def test_gradient_descent_256_options(cuda, potential, masked, fix_probe):
    st = make_state(S=256, J=12, potential=potential, seed=257 + int(potential))
    mask = None
    if masked:
        mask = (np.random.default_rng(5).uniform(size=(256, 256)) > 0.05).astype(np.float32)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=2, max_batch_size=5, seed_random=2,
            detector_fourier_mask=mask, fix_probe=fix_probe, **OFF)


@pytest.mark.parametrize("modes,slices", [(2, 1), (1, 2), (2, 2)])
def test_mixed_and_multislice_256(cuda, modes, slices):
    st = make_state(S=256, J=9, modes=modes, slices=slices, seed=300 + 10 * modes + slices)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=5, seed_random=3, **OFF)


def resampled_state(state, detector, seed):
    """The state's model with the far field resampled onto a `detector` grid:
    the amplitudes are Poisson counts (0.05 per unit intensity, as make_state's)
    of the oracle's float64 resampled far field of a perturbed object, so the
    data follow the resampling model and the dark field is exactly zero (where
    the far field is tiny but not zero, A exp(i angle F) takes a phase set by
    rounding and float32 and float64 evaluations part by 1e-3)."""
    import dataclasses

    rng = np.random.default_rng(seed)
    s = dataclasses.replace(state, roi_shape=tuple(state.amplitudes.shape[-2:]),
                            resample_exit_waves=True)
    o = Oracle(s, "float64")
    o.amp_shape = np.array(detector)
    truth = o.object * np.exp(1j * rng.uniform(-0.05, 0.05, o.object.shape))
    o.object = truth
    pos = o.positions_px
    frac = pos - np.round(pos)
    rows, cols = o.patch_indices(pos)
    shifted = o.fft_shift(o.probe, frac)
    _, _, ov = o.overlap(rows, cols, shifted)
    inten = o.farfield(o.to_detector(o.fft2(ov))) ** 2
    amps = np.sqrt(rng.poisson(inten * 0.05) / 0.05).astype(np.float32)
    return dataclasses.replace(s, amplitudes=amps)


@pytest.mark.parametrize("S,detector,modes", [(64, (48, 48), 1), (48, (64, 64), 1),
                                              (64, (96, 80), 2), (96, (64, 64), 1)])
def test_resampled_far_field(cuda, S, detector, modes):
    """region_of_interest_shape: the far field is resampled to the detector grid
    and back (staged path at a fused size), against the oracle. When the
    detector grid is coarser than the ROI's, linear interpolation of the complex
    far field makes near-zeros between samples of differing phase, where
    A exp(i angle F) follows the rounding of F, so any change of the float32
    FFT's rounding moves the result far more than elsewhere: the oracle with
    every FFT through complex128 (another float32 FFT) lies 1e-5 - 1e-3 from it
    (the floor, measured here), and a third float32 FFT, the GPU's, lands a few
    floors away. Bar: 2e-5, or 10x the floor where that is larger. (A float32
    emulation of these kernels with the oracle's own FFT agrees with the oracle
    to 1e-6.)"""
    st = resampled_state(make_state(S=S, J=12, modes=modes, seed=400 + S), detector, S)
    kw = dict(num_iter=2, max_batch_size=5, seed_random=4, **OFF)
    o = Oracle(st).reconstruct(**kw)
    rt = Oracle(st, fft_round_trip=True).reconstruct(**kw)
    g_obj, g_probe, g_err = gpu_reconstruct(st, **kw)

    def err_rel(x, y):
        x, y = np.array(x), np.array(y)
        return float(np.max(np.abs(x - y) / np.abs(y)))

    for name, d, floor in (("object", rel(g_obj, o.object), rel(rt.object, o.object)),
                           ("probe", rel(g_probe, o.probe), rel(rt.probe, o.probe)),
                           ("error", err_rel(g_err, o.error_iterations),
                            err_rel(rt.error_iterations, o.error_iterations))):
        print(f"{name} {d:.2e} (floor {floor:.2e})")
        assert d < max(2e-5, 10 * floor), (name, d, floor)


def test_constraints_256(cuda):
    """Default constraints: probe centre of mass (staged probe shift), the
    potential baseline and object positivity, three iterations."""
    st = make_state(S=256, J=16, seed=259)
    compare(st, 1e-4, 1e-4, 2e-5, num_iter=3, max_batch_size=6, seed_random=5)


def test_self_consistency_256(cuda):
    from py4dstem_gb300 import engine

    st = make_state(S=256, J=10, seed=260)
    ref = Oracle(st).self_consistency_errors(max_batch_size=4)
    dev = engine.create_state(
        roi_shape=(256, 256), object_array=st.object, probe_array=st.probe,
        amplitudes=st.amplitudes, positions_px=st.positions_px, num_slices=1, num_probes=1,
        potential=False, max_batch=4)
    got = engine.self_consistency_errors(dev, 4).astype(np.float64) / st.mean_intensity
    d = np.max(np.abs(got - ref) / ref)
    print(f"self-consistency max rel {d:.2e}")
    assert d < 2e-5, d


def test_probe_aperture_256(cuda):
    import torch

    from py4dstem_gb300 import _native

    lib = _native.lib()
    st = make_state(S=256, J=4, seed=261)
    rng = np.random.default_rng(3)
    probe = (st.probe * np.exp(1j * rng.uniform(-0.3, 0.3, st.probe.shape))).astype(np.complex64)
    aperture = np.abs(np.fft.fft2(st.probe)).astype(np.float32)
    ref = Oracle._probe_aperture(probe.astype(np.complex128), aperture.astype(np.float64))
    g = _native.Geometry(256, 256, 320, 320, 1, 1, 0, 0)
    p = torch.from_numpy(probe).cuda()
    a = torch.from_numpy(aperture).cuda()
    _native.check(lib.ptycho_probe_aperture_constraint(
        ctypes.byref(g), ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(a.data_ptr()), None))
    torch.cuda.synchronize()
    d = rel(p.cpu().numpy(), ref)
    print(f"aperture rel {d:.2e}")
    assert d < 1e-5, d


def test_object_gradient_256(cuda):
    """ptycho_gd_gradient at 256^2: dloss/dO = -2N scatter(conj(P) chi) of the
    whole scan (float32 oracle), the loss is the batch error; the probe gradient
    is refused."""
    import torch

    from py4dstem_gb300.autograd import PtychoForwardModel

    state = make_state(S=256, J=6, seed=262)
    model = PtychoForwardModel(state.amplitudes, state.positions_px, np.shape(state.object)[-2:],
                               max_batch=4)
    obj = torch.tensor(np.asarray(state.object), device="cuda")
    probe = torch.tensor(np.asarray(state.probe, np.complex64)[None], device="cuda")
    loss, g_obj, g_probe = model.loss_and_gradient(obj, probe, probe_gradient=False)
    assert g_probe is None
    def oracle_terms(o):
        idx = np.arange(o.J)
        shifted, patches, _, chi, err = o.forward_batch(idx)
        return o.scatter(o._obj_term(patches, shifted, chi), o.positions_px[idx]), err

    term, err = oracle_terms(Oracle(state))
    # the reference algorithm's own rounding floor here: the same model with
    # every FFT through complex128 (the dark field's phase is rounding-determined)
    floor = rel(oracle_terms(Oracle(state, fft_round_trip=True))[0], term)
    term64 = oracle_terms(Oracle(state, "float64"))[0]
    N = 256 * 256
    d_grad = rel(g_obj.cpu().numpy(), -2 * N * term)
    d_loss = abs(float(loss) - float(err)) / float(err)
    print(f"grad {d_grad:.2e} (floor {floor:.2e}, vs FP64 "
          f"{rel(g_obj.cpu().numpy(), -2 * N * term64):.2e}) loss {d_loss:.2e}")
    assert d_grad < max(1e-5, 3 * floor) and d_loss < 1e-5
    with pytest.raises(RuntimeError, match="probe gradient is not available"):
        model.loss_and_gradient(obj, probe, probe_gradient=True)
