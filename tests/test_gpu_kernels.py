"""GPU parity of the fused kernels against the oracle on small seeded states.

One or a few iterations from a non-uniform initial object, where the reference
algorithm is well conditioned, so the GPU must agree with the float32 oracle to
a few float32 ulps amplified by the iteration (tolerances written per test)."""

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
    return g_obj, g_probe, g_err


@pytest.mark.parametrize("S", [32, 48, 64, 96, 128])
def test_single_slice_one_iteration(cuda, S):
    st = make_state(S=S, J=25, seed=S)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=13, seed_random=1, **OFF)


@pytest.mark.parametrize("potential,masked,fix_probe", [(True, False, False), (False, True, False),
                                                        (False, False, True)])
def test_register_resident_128_variants(cuda, potential, masked, fix_probe):
    """The 128^2 single-slice kernel (register-resident FFT) with each option."""
    from py4dstem_gb300 import _native

    lib = _native.lib()
    st = make_state(S=128, J=20, potential=potential, seed=21)
    mask = None
    if masked:
        mask = (np.random.default_rng(1).uniform(size=(128, 128)) > 0.05).astype(np.float32)
    lib.ptycho_set_kernel_schedule(128, 2)
    try:
        compare(st, 2e-5, 2e-5, 2e-5, num_iter=2, max_batch_size=7, seed_random=2,
                detector_fourier_mask=mask, fix_probe=fix_probe, **OFF)
    finally:
        lib.ptycho_set_kernel_schedule(128, 0)


@pytest.mark.parametrize("potential,masked,fix_probe", [
    (False, False, False), (True, False, False), (False, True, False), (False, False, True)])
def test_grouped_128_variants(cuda, potential, masked, fix_probe):
    """The 128^2 single-slice kernel with passes by groups of warps (schedule 3)
    with each option, against the oracle and against the block-wide schedule."""
    from py4dstem_gb300 import _native

    lib = _native.lib()
    st = make_state(S=128, J=20, potential=potential, seed=27)
    mask = None
    if masked:
        mask = (np.random.default_rng(3).uniform(size=(128, 128)) > 0.05).astype(np.float32)
    kw = dict(num_iter=2, max_batch_size=7, seed_random=5, detector_fourier_mask=mask,
              fix_probe=fix_probe, **OFF)
    try:
        lib.ptycho_set_kernel_schedule(128, 3)
        g = compare(st, 2e-5, 2e-5, 2e-5, **kw)
        lib.ptycho_set_kernel_schedule(128, 1)
        b = gpu_reconstruct(st, **kw)
    finally:
        lib.ptycho_set_kernel_schedule(128, 0)
    assert rel(g[0], b[0]) < 2e-6
    assert rel(g[1], b[1]) < 2e-6


@pytest.mark.parametrize("slices,potential,masked", [(3, False, False), (2, True, False),
                                                      (4, False, True)])
def test_grouped_128_multislice(cuda, slices, potential, masked):
    """Multislice gradient descent at 128^2 with passes by groups of warps (the
    default schedule), against the oracle and the block-wide schedule."""
    from py4dstem_gb300 import _native

    lib = _native.lib()
    st = make_state(S=128, J=12, slices=slices, potential=potential, seed=81 + slices)
    mask = None
    if masked:
        mask = (np.random.default_rng(9).uniform(size=(128, 128)) > 0.05).astype(np.float32)
    kw = dict(num_iter=2, max_batch_size=5, seed_random=7, detector_fourier_mask=mask, **OFF)
    try:
        lib.ptycho_set_kernel_schedule(128, 3)
        g = compare(st, 2e-5, 2e-5, 2e-5, **kw)
        lib.ptycho_set_kernel_schedule(128, 1)
        b = gpu_reconstruct(st, **kw)
    finally:
        lib.ptycho_set_kernel_schedule(128, 0)
    assert rel(g[0], b[0]) < 2e-6
    assert rel(g[1], b[1]) < 2e-6


@pytest.mark.parametrize("modes,masked", [(3, False), (2, True), (1, False)])
def test_grouped_128_mixed_state(cuda, modes, masked):
    """Mixed-state single-slice gradient descent at 128^2 with passes by groups
    of warps (one mode: the mixed-state formula on a single probe), against the
    oracle and the block-wide schedule."""
    from py4dstem_gb300 import _native

    lib = _native.lib()
    st = make_state(S=128, J=12, modes=modes, seed=85 + modes)
    if modes == 1:
        st.mixed = True
        st.probe = st.probe[None]
    mask = None
    if masked:
        mask = (np.random.default_rng(11).uniform(size=(128, 128)) > 0.05).astype(np.float32)
    kw = dict(num_iter=2, max_batch_size=5, seed_random=8, detector_fourier_mask=mask, **OFF)
    try:
        lib.ptycho_set_kernel_schedule(128, 3)
        g = compare(st, 2e-5, 2e-5, 2e-5, **kw)
        lib.ptycho_set_kernel_schedule(128, 1)
        b = gpu_reconstruct(st, **kw)
    finally:
        lib.ptycho_set_kernel_schedule(128, 0)
    assert rel(g[0], b[0]) < 2e-6
    assert rel(g[1], b[1]) < 2e-6


@pytest.mark.parametrize("slices,modes,potential", [(2, 2, False), (3, 3, True)])
def test_grouped_128_mixed_state_multislice(cuda, slices, modes, potential):
    """Mixed-state multislice gradient descent at 128^2 with passes by groups of
    warps, against the oracle and the block-wide schedule."""
    from py4dstem_gb300 import _native

    lib = _native.lib()
    st = make_state(S=128, J=10, slices=slices, modes=modes, potential=potential,
                    seed=70 + slices + modes)
    kw = dict(num_iter=2, max_batch_size=4, seed_random=6, **OFF)
    try:
        lib.ptycho_set_kernel_schedule(128, 3)
        g = compare(st, 2e-5, 2e-5, 2e-5, **kw)
        lib.ptycho_set_kernel_schedule(128, 1)
        b = gpu_reconstruct(st, **kw)
    finally:
        lib.ptycho_set_kernel_schedule(128, 0)
    assert rel(g[0], b[0]) < 2e-6
    assert rel(g[1], b[1]) < 2e-6


def test_both_128_schedules_agree_with_oracle(cuda):
    """Shared-memory passes (block-wide and by groups of warps) and the
    register-resident schedule at 128^2."""
    from py4dstem_gb300 import _native

    lib = _native.lib()
    st = make_state(S=128, J=16, seed=23)
    try:
        for schedule in (1, 2, 3):
            lib.ptycho_set_kernel_schedule(128, schedule)
            compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=8, seed_random=4, **OFF)
    finally:
        lib.ptycho_set_kernel_schedule(128, 0)


@pytest.mark.parametrize("S", [(96, 128), (128, 96)])
def test_non_square_roi(cuda, S):
    """Non-square regions of interest (a 96 x 128 detector either way round):
    gradient descent, then a mixed state and a multislice model, one iteration
    each against the oracle."""
    st = make_state(S=S, J=16, seed=sum(S))
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=8, seed_random=1, **OFF)
    st = make_state(S=S, J=16, modes=2, seed=sum(S) + 1)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=8, seed_random=2, **OFF)
    st = make_state(S=S, J=16, slices=2, seed=sum(S) + 2)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=8, seed_random=3, **OFF)
    # the probe centre-of-mass constraint shifts non-square probes too
    st = make_state(S=S, J=16, seed=sum(S) + 3)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=2, max_batch_size=8, seed_random=4,
            fix_potential_baseline=False, orthogonalize_probe=False)


def test_potential_object(cuda):
    st = make_state(S=64, J=25, potential=True, seed=3)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=9, seed_random=2, **OFF)


@pytest.mark.parametrize("modes", [2, 3])
def test_mixed_state(cuda, modes):
    st = make_state(S=64, J=25, modes=modes, seed=4)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=10, seed_random=3, **OFF)


def test_mixed_formula_single_mode(cuda):
    st = make_state(S=32, J=16, modes=1, seed=5)
    st.mixed = True
    st.probe = st.probe[None]
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=8, seed_random=3, **OFF)


@pytest.mark.parametrize("slices,potential", [(2, False), (3, False), (2, True)])
def test_multislice(cuda, slices, potential):
    st = make_state(S=64, J=16, slices=slices, potential=potential, seed=6 + slices)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=8, seed_random=4, **OFF)


@pytest.mark.parametrize("S,slices,modes,potential", [(64, 2, 2, False), (32, 3, 3, False),
                                                      (64, 2, 2, True), (128, 2, 2, False),
                                                      (96, 3, 2, False)])
def test_mixed_state_multislice(cuda, S, slices, modes, potential):
    """Every probe mode through every slice (kernel mode 4), two iterations."""
    st = make_state(S=S, J=16, slices=slices, modes=modes, potential=potential,
                    seed=40 + S + slices + modes)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=2, max_batch_size=8, seed_random=5, **OFF)


def test_mixed_state_multislice_mask_fix_probe_constraints(cuda):
    st = make_state(S=64, J=16, slices=2, modes=2, seed=47)
    mask = (np.random.default_rng(3).uniform(size=(64, 64)) > 0.05).astype(np.float32)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=2, max_batch_size=8, seed_random=6,
            detector_fourier_mask=mask, fix_probe=True, **OFF)
    # with the per-iteration constraints (mode orthogonalisation amplifies rounding
    # in the weak modes) the bar of test_constraints_several_iterations
    st = make_state(S=64, J=16, slices=2, modes=3, seed=48)
    compare(st, 1e-4, 1e-4, 2e-5, num_iter=3, max_batch_size=8, seed_random=7,
            fix_probe_com=True, fix_potential_baseline=True, orthogonalize_probe=True)


@pytest.mark.parametrize("abc", [(-1.0, 1.0, 2.0), (0.0, 0.5, 2.0), (0.3, 0.6, 1.4)])
def test_mixed_state_multislice_projection_sets(cuda, abc):
    """Projection sets through kernel mode 4: per-mode exit waves at the last slice."""
    st = make_state(S=32, J=16, slices=2, modes=2, seed=49)
    a, b, c = abc
    compare(st, 5e-5, 5e-5, 5e-5, num_iter=2, method="PS", a=a, b=b, c=c, **OFF)


@pytest.mark.parametrize("method,abc", [("DM", (-1.0, 1.0, 2.0)), ("RAAR", (0.0, 0.5, 2.0)),
                                        ("RRR", (-1.0, 1.0, 2.0)), ("SUPERFLIP", (0.0, 1.0, 2.0)),
                                        ("GP", (0.3, 0.6, 1.4))])
def test_projection_sets(cuda, method, abc):
    st = make_state(S=32, J=16, seed=7)
    a, b, c = abc
    compare(st, 5e-5, 5e-5, 5e-5, num_iter=2, method="PS", a=a, b=b, c=c, **OFF)


@pytest.mark.parametrize("abc,potential", [((-1.0, 1.0, 2.0), False), ((0.0, 0.5, 2.0), True),
                                           ((0.3, 0.6, 1.4), False)])
def test_grouped_128_projection_sets(cuda, abc, potential):
    """Projection sets (DM, RAAR, generalized) at 128^2 with passes by groups of
    warps, against the oracle and the block-wide schedule."""
    from py4dstem_gb300 import _native

    lib = _native.lib()
    st = make_state(S=128, J=12, potential=potential, seed=95 + int(10 * abc[1]))
    a, b, c = abc
    kw = dict(num_iter=3, method="PS", a=a, b=b, c=c, **OFF)
    try:
        lib.ptycho_set_kernel_schedule(128, 3)
        g = compare(st, 5e-5, 5e-5, 5e-5, **kw)
        lib.ptycho_set_kernel_schedule(128, 1)
        bw = gpu_reconstruct(st, **kw)
    finally:
        lib.ptycho_set_kernel_schedule(128, 0)
    assert rel(g[0], bw[0]) < 1e-5
    assert rel(g[1], bw[1]) < 1e-5


def test_projection_mixed_and_multislice(cuda):
    st = make_state(S=32, J=16, modes=2, seed=8)
    compare(st, 5e-5, 5e-5, 5e-5, num_iter=2, method="PS", a=0.0, b=0.5, c=2.0, **OFF)
    st = make_state(S=32, J=16, slices=2, seed=9)
    compare(st, 5e-5, 5e-5, 5e-5, num_iter=2, method="PS", a=-1.0, b=1.0, c=2.0, **OFF)


def test_fix_probe_and_detector_mask(cuda):
    st = make_state(S=64, J=16, seed=10)
    mask = (np.random.default_rng(0).uniform(size=(64, 64)) > 0.1).astype(np.float32)
    compare(st, 2e-5, 2e-5, 2e-5, num_iter=1, max_batch_size=8, seed_random=1, fix_probe=True,
            detector_fourier_mask=mask, **OFF)


def test_constraints_several_iterations(cuda):
    st = make_state(S=64, J=25, seed=11)
    compare(st, 1e-4, 1e-4, 2e-5, num_iter=4, max_batch_size=9, seed_random=5)
    st = make_state(S=64, J=25, seed=12, potential=True)
    compare(st, 1e-4, 1e-4, 2e-5, num_iter=3, max_batch_size=9, seed_random=5, shrinkage_rad=0.01)
    st = make_state(S=32, J=16, modes=3, seed=13)
    compare(st, 1e-4, 1e-4, 2e-5, num_iter=3, max_batch_size=8, seed_random=5)
    st = make_state(S=32, J=16, seed=14)
    compare(st, 1e-4, 1e-4, 2e-5, num_iter=3, max_batch_size=8, seed_random=5,
            pure_phase_object=True)


def test_deterministic_and_storage_independent(cuda):
    st = make_state(S=64, J=25, seed=15)
    kw = dict(num_iter=2, max_batch_size=7, seed_random=9)
    a = gpu_reconstruct(st, **kw)
    b = gpu_reconstruct(st, **kw)
    c = gpu_reconstruct(st, storage="cpu", **kw)
    for x, y in ((a, b), (a, c)):
        np.testing.assert_array_equal(x[0], y[0])
        np.testing.assert_array_equal(x[1], y[1])
        assert x[2] == y[2]


@pytest.mark.parametrize("J,B", [(1, 1), (7, 3), (2100, 2100), (2100, 700)])
def test_batch_edges(cuda, J, B):
    """A single position; ragged batches; a batch longer than the object
    reduction's 2048-position list window (two windows per tile)."""
    st = make_state(S=32, J=J, seed=60 + J % 7, obj_px=None if J < 100 else 192)
    tol = 2e-5 if J < 100 else 5e-5
    compare(st, tol, tol, tol, num_iter=2, max_batch_size=B, seed_random=3, **OFF)


@pytest.mark.parametrize("shape,potential,pure_phase,sigma", [
    ((1, 96, 80), False, False, 1.7), ((3, 64, 64), True, False, 0.9),
    ((2, 40, 56), False, True, 2.4), ((1, 48, 48), False, False, 20.0)])
def test_object_gaussian_matches_scipy(cuda, shape, potential, pure_phase, sigma):
    """The object blur against scipy.ndimage.gaussian_filter (reflecting edges,
    every axis of the object array; a radius larger than the object too)."""
    import ctypes

    import torch
    from scipy.ndimage import gaussian_filter

    from py4dstem_gb300 import _native, engine

    rng = np.random.default_rng(int(sigma * 10) + shape[0])
    if potential:
        obj = rng.normal(size=shape).astype(np.float32)
    else:
        obj = (np.exp(1j * rng.normal(size=shape)) * (1 + 0.1 * rng.normal(size=shape))
               ).astype(np.complex64)
    ref = obj[0] if shape[0] == 1 else obj
    if pure_phase:
        ref = np.exp(1.0j * gaussian_filter(np.angle(ref), sigma))
    else:
        ref = gaussian_filter(ref, sigma)
    radius = int(4.0 * sigma + 0.5)
    x = np.arange(-radius, radius + 1)
    w = np.exp(-0.5 / (sigma * sigma) * x ** 2)
    w = w / w.sum()
    g = engine.make_geometry((32, 32), shape[1:], shape[0], 1, potential)
    o = torch.from_numpy(obj).cuda()
    wd = torch.from_numpy(w).cuda()
    scratch = torch.empty(4 * o.numel(), dtype=torch.float32, device="cuda")
    _native.check(_native.lib().ptycho_object_gaussian_constraint(
        ctypes.byref(g), ctypes.c_void_p(o.data_ptr()), ctypes.c_void_p(wd.data_ptr()), radius,
        1 if pure_phase else 0, ctypes.c_void_p(scratch.data_ptr()), None))
    got = o.cpu().numpy().reshape(np.shape(ref))
    assert np.max(np.abs(got - ref)) <= 2e-6 * np.max(np.abs(ref))
