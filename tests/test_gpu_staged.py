"""The 256 x 256 region of interest (batch-wide staged kernels) against the
oracle: gradient descent with each option, the constraints over several
iterations, the forward-only errors, the probe aperture constraint and the
object gradient. Tolerances as for the fused kernels (the 256-point transforms
round like the 128-point ones: two radix-16 passes)."""

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
    o = Oracle(state)
    idx = np.arange(o.J)
    shifted, patches, _, chi, err = o.forward_batch(idx)
    term = o.scatter(o._obj_term(patches, shifted, chi), o.positions_px[idx])
    N = 256 * 256
    d_grad = rel(g_obj.cpu().numpy(), -2 * N * term)
    d_loss = abs(float(loss) - float(err)) / float(err)
    print(f"grad {d_grad:.2e} loss {d_loss:.2e}")
    assert d_grad < 1e-5 and d_loss < 1e-5
    with pytest.raises(RuntimeError, match="probe gradient is not available"):
        model.loss_and_gradient(obj, probe, probe_gradient=True)
