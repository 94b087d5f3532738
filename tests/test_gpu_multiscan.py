"""Many scans in one graph-captured, concurrent launch (py4dstem_gb300.multiscan).

Each scan of a multi-scan run must give, bit for bit, what a reconstruction of
that scan alone gives with the same position orders (RandomState(seed + k)) and
the same device-side mixed-state orthogonalisation: concurrency and graph replay
change the schedule, never the arithmetic. The device orthogonalisation equals
the host (LAPACK) one up to one phase per mode.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scans():
    from py4dstem_gb300 import MixedstatePtychography, SingleslicePtychography, synthetic

    specs = [
        dict(name="a", seed=21, scan_shape=(8, 8), step_ang=0.5, jitter_ang=0.05, detector=64,
             object_px=96, num_modes=2, mode_weights=(0.8, 0.2)),
        dict(name="b", seed=22, scan_shape=(6, 9), step_ang=0.5, jitter_ang=0.05, detector=96,
             object_px=128),
        dict(name="c", seed=23, scan_shape=(10, 7), step_ang=0.5, jitter_ang=0.05, detector=64,
             object_px=96, num_modes=3, mode_weights=(0.7, 0.2, 0.1)),
    ]
    out = []
    for sp in specs:
        case = synthetic.make_scan(**sp)
        kw = dict(case.ctor_kwargs)
        cls = MixedstatePtychography if sp.get("num_modes", 1) > 1 else SingleslicePtychography
        if case.probe_modes is not None:
            kw["initial_probe_guess"] = case.probe_modes.astype(np.complex64)
        p = cls(datacube=case.datacube, verbose=False, device="gpu", **kw)
        p.preprocess(**case.preprocess_kwargs)
        out.append(p)
    return out


def _alone(p, k, seed, num_iter, batch):
    """One scan through the engine directly: the same orders and options."""
    from py4dstem_gb300 import engine

    potential = p._object_type == "potential"
    st = engine.create_state(
        roi_shape=tuple(p._region_of_interest_shape), object_array=np.asarray(p._object),
        probe_array=p._probe, amplitudes=p._amplitudes, positions_px=p._positions_px,
        num_slices=p._num_slices, num_probes=p._num_probes, potential=potential,
        max_batch=batch, storage="gpu",
        fov_mask_inverse=p._object_fov_mask_inverse, mixed_state=p._mixed)
    drv = engine.IterationDriver(
        st, max_batch=batch, use_mask=bool(p._object_fov_mask_inverse.sum() > 0),
        orthogonalize_probe=True, mean_intensity=p._mean_diffraction_intensity,
        device_orthogonalization=True)
    rng = np.random.RandomState(seed + k)
    order = np.arange(p._num_diffraction_patterns)
    errors = []
    for _ in range(num_iter):
        rng.shuffle(order)
        drv.iterate(order)
        errors.append(float(drv.error()))
    return st.object.cpu().numpy(), st.probe.cpu().numpy(), errors


@pytest.mark.parametrize("use_graph,concurrent", [(True, "auto"), (True, False), (False, True)])
def test_multiscan_equals_each_scan_alone(cuda, use_graph, concurrent):
    from py4dstem_gb300.multiscan import MultiScanReconstruction

    scans = _scans()
    refs = [_alone(p, k, 5, 4, 16) for k, p in enumerate(scans)]
    run = MultiScanReconstruction(scans, max_batch_size=16, seed_random=5,
                                  use_graph=use_graph, concurrent=concurrent)
    run.reconstruct(4)
    for p, (obj, probe, errors) in zip(scans, refs):
        np.testing.assert_array_equal(p._object, obj)
        np.testing.assert_array_equal(np.asarray(p._probe).reshape(probe.shape), probe)
        np.testing.assert_allclose(p.error_iterations, errors, rtol=0, atol=0)
    if concurrent == "auto":
        assert run.tuning["choice"]["concurrent"] in (True, False)
        assert len(run.tuning["timings_ms"]) == 2


def test_device_orthogonalization_matches_host_up_to_phase(cuda):
    torch = cuda
    from py4dstem_gb300 import engine

    rng = np.random.default_rng(3)
    M, S = 4, 64
    probe = (rng.normal(size=(M, S, S)) + 1j * rng.normal(size=(M, S, S))).astype(np.complex64)
    probe *= np.array([3.0, 1.0, 0.5, 0.2], np.float32)[:, None, None]

    def state():
        return engine.create_state(
            roi_shape=(S, S), object_array=np.ones((96, 96), np.complex64), probe_array=probe,
            amplitudes=np.ones((1, S, S), np.float32),
            positions_px=np.full((1, 2), 48.0, np.float32), num_slices=1, num_probes=M,
            potential=False, max_batch=1, storage="gpu")

    a, b = state(), state()
    engine.probe_orthogonalization(a, on_device=False)
    engine.probe_orthogonalization(b, on_device=True)
    torch.cuda.synchronize()
    pa = a.probe.cpu().numpy().reshape(M, -1).astype(np.complex128)
    pb = b.probe.cpu().numpy().reshape(M, -1).astype(np.complex128)
    for m in range(M):
        c = np.vdot(pa[m], pb[m]) / (np.linalg.norm(pa[m]) * np.linalg.norm(pb[m]))
        assert abs(abs(c) - 1.0) < 1e-5  # same mode up to a phase
    # modes are orthogonal and ordered by decreasing intensity
    gram = pb.conj() @ pb.T
    off = gram - np.diag(np.diag(gram))
    assert np.abs(off).max() < 1e-4 * np.abs(np.diag(gram)).max()
    inten = np.real(np.diag(gram))
    assert np.all(np.diff(inten) <= 0)
