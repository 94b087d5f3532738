"""Host-resident amplitudes gathered to the device one batch ahead.

With page-locked host amplitudes every batch's patterns are gathered into one of
two device slots by ptycho_gather_patterns on a second stream while the batch
before it computes. The batch kernels then read the same values as with
device-resident amplitudes, so whole reconstructions must agree bit for bit,
eagerly and under CUDA-graph replay, on ragged batch splits."""

import ctypes

import numpy as np
import pytest

from gpu_helpers import make_state

pytestmark = pytest.mark.gpu


def _pinned(arr):
    import torch

    t = torch.empty(arr.shape, dtype=torch.float32, pin_memory=True)
    t.numpy()[...] = arr
    return t


@pytest.mark.parametrize("size,offset", [(256, 0), (143, 0), (256, 1)])
@pytest.mark.parametrize("source", ["device", "host"])
def test_gather_patterns_exact(cuda, size, offset, source):
    """out[i] = patterns[rows[i]] bit for bit: 16-byte vectors (256 values) and
    the scalar form (143 values, or a source one float off 16-byte alignment);
    rows outside [0, J) give NaN rows; device or page-locked host source."""
    import torch

    from py4dstem_gb300 import _native, engine

    lib = _native.lib()
    J, n = 37, 29
    rng = np.random.default_rng(size + offset)
    src = rng.normal(size=(J * size + offset,)).astype(np.float32)
    rows = rng.integers(0, J, n).astype(np.int32)
    rows[3], rows[17] = -1, J
    if source == "device":
        src_t = torch.from_numpy(src).cuda()
        base = src_t.data_ptr()
    else:
        src_t = _pinned(src)
        base = engine.mapped_host_address(src_t.numpy())
        assert base is not None
    rows_t = torch.from_numpy(rows).cuda()
    out = torch.full((n, size), 7.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    _native.check(lib.ptycho_gather_patterns(
        ctypes.c_void_p(base + 4 * offset), J, size, ctypes.c_void_p(rows_t.data_ptr()), n,
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream)))
    got = out.cpu().numpy()
    table = src[offset:].reshape(J, size)
    for i, r in enumerate(rows):
        if 0 <= r < J:
            np.testing.assert_array_equal(got[i], table[r])
        else:
            assert np.all(np.isnan(got[i]))
    # no row list: the first n patterns
    out2 = torch.empty((n, size), dtype=torch.float32, device="cuda")
    _native.check(lib.ptycho_gather_patterns(
        ctypes.c_void_p(base + 4 * offset), J, size, None, n, ctypes.c_void_p(out2.data_ptr()),
        ctypes.c_void_p(stream)))
    np.testing.assert_array_equal(out2.cpu().numpy(), table[:n])


def _run(state, amplitudes, storage, *, graph, iters, batch, projection=False, seed=5):
    from py4dstem_gb300 import engine

    J = state.amplitudes.shape[0]
    st = engine.create_state(
        roi_shape=state.amplitudes.shape[-2:], object_array=state.object,
        probe_array=state.probe, amplitudes=amplitudes, positions_px=state.positions_px,
        num_slices=state.num_slices, num_probes=state.num_probes,
        potential=state.object_type == "potential", max_batch=batch, storage=storage,
        propagators=state.propagators, projection=projection, mixed_state=state.mixed)
    assert (st.amp_ring is not None) == (storage == "cpu")
    drv = engine.IterationDriver(
        st, max_batch=batch, projection=projection, step_size=0.5,
        projection_abc=(0.0, 1.0, 0.0) if projection else (0.0, 0.0, 0.0),
        fix_probe_com=True, mean_intensity=state.mean_intensity, graph=graph)
    rng = np.random.default_rng(seed)
    errors = []
    for _ in range(iters):
        order = rng.permutation(J) if not projection else np.arange(J)
        drv.iterate(order)
        errors.append(float(drv.error()))
    if graph:
        assert drv.graph is not None
    return st.object.cpu().numpy(), st.probe.cpu().numpy(), errors


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("J,B", [(25, 7), (9, 2), (30, 30)])
def test_prefetched_host_amplitudes_match_resident(cuda, graph, J, B):
    state = make_state(S=64, J=J, seed=70 + J)
    pinned = _pinned(state.amplitudes)
    a = _run(state, state.amplitudes, "gpu", graph=graph, iters=4, batch=B)
    b = _run(state, pinned.numpy(), "cpu", graph=graph, iters=4, batch=B)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2] == b[2]


def test_prefetched_host_amplitudes_mixed_multislice_projection(cuda):
    """Projection sets (exit waves kept per position) on a mixed-state
    multislice state, three batches, graph replay."""
    state = make_state(S=32, J=20, modes=2, slices=2, seed=91)
    pinned = _pinned(state.amplitudes)
    a = _run(state, state.amplitudes, "gpu", graph=True, iters=3, batch=7, projection=True)
    b = _run(state, pinned.numpy(), "cpu", graph=True, iters=3, batch=7, projection=True)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2] == b[2]


def test_grouped_kernel_amplitude_sources_agree(cuda):
    """The 128^2 grouped schedule on device amplitudes and on page-locked host
    rows that the kernel reads in place (the C ABI takes either): the same bits."""
    from py4dstem_gb300 import _native, engine

    lib = _native.lib()
    state = make_state(S=128, J=12, seed=93)
    pinned = _pinned(state.amplitudes)
    try:
        lib.ptycho_set_kernel_schedule(128, 3)
        a = _run(state, state.amplitudes, "gpu", graph=False, iters=2, batch=5)
        st = engine.create_state(
            roi_shape=(128, 128), object_array=state.object, probe_array=state.probe,
            amplitudes=pinned.numpy(), positions_px=state.positions_px, num_slices=1,
            num_probes=1, potential=False, max_batch=5, storage="cpu")
        st.amp_ring = None  # in-place reads of the mapped host rows
        drv = engine.IterationDriver(st, max_batch=5, step_size=0.5, fix_probe_com=True,
                                     mean_intensity=state.mean_intensity)
        rng = np.random.default_rng(5)
        errors = []
        for _ in range(2):
            drv.iterate(rng.permutation(12))
            errors.append(float(drv.error()))
    finally:
        lib.ptycho_set_kernel_schedule(128, 0)
    np.testing.assert_array_equal(a[0], st.object.cpu().numpy())
    np.testing.assert_array_equal(a[1], st.probe.cpu().numpy())
    assert a[2] == errors


def test_prefetched_host_amplitudes_with_position_correction(cuda):
    """Gradient descent with position correction through the public API: the
    correction reads the batch's gathered rows from the same device slot."""
    from golden_io import Golden

    g = Golden("ss_gd_poscorr")
    out = []
    for storage in ("gpu", "cpu"):
        p = g.build(storage=storage)
        if storage == "cpu":
            p._amplitudes = _pinned(np.ascontiguousarray(p._amplitudes)).numpy()
        p.reconstruct(progress_bar=False, **g.rec_kwargs())
        out.append((np.asarray(p._object), np.asarray(p._probe), list(p.error_iterations),
                    np.array(p._positions_px)))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]
    np.testing.assert_array_equal(out[0][3], out[1][3])
