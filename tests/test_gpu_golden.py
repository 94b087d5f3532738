"""End-to-end parity of the drop-in classes against the unmodified reference.

Each golden fixture is reconstructed through the public API (constructor,
preprocess(), reconstruct()) on the GPU and compared with what the reference's
CPU path returned on the same datacube, seed and arguments.

Tolerances. The reference itself is sensitive to floating-point rounding: with a
uniform initial object the far field of the first iteration is exactly zero
outside the probe aperture, so A*exp(i*angle(F)) takes a rounding-determined
phase there; projection-set methods (RAAR here) are chaotic on small scans. We
measure that floor by re-running the oracle with every FFT evaluated in
complex128 and rounded back to complex64 (a different, correct float32 FFT).
Gradient-descent fixtures must meet the parity tolerance outright (error per
iteration 1e-5 relative, object and probe 1e-4 relative L2); the one whose
measured floor is at that bar already (FLOOR_BOUND) takes 3x the floor.
Projection-set fixtures take 5x the floor. Each result's distance to the
float64 evaluation of the same model is printed.
"""

import numpy as np
import pytest

from golden_io import Golden, names, rel_l2
from oracle.ptycho_np import Oracle

pytestmark = pytest.mark.gpu

# Gradient-descent fixtures meet the parity bar outright (error 1e-5 per
# iteration, object and probe 1e-4), except where the reference's own rounding
# floor is at that bar already: there 3x the floor.
FLOOR_BOUND = {
    # mixed state with position correction: the probe floor is 1.3e-4 (the
    # reference moves by that much under another float32 FFT)
    "mixed_gd_poscorr",
}


@pytest.mark.parametrize("name", names())
def test_reconstruction_matches_reference(cuda, name):
    g = Golden(name)
    p = g.build(device="gpu")
    state = g.state(p)
    kw = g.oracle_kwargs()
    p.reconstruct(progress_bar=False, **g.rec_kwargs())

    ref_err = g.out["error_iterations"]
    err = np.asarray(p.error_iterations)
    d_err = float(np.max(np.abs(err - ref_err) / np.abs(ref_err)))
    d_obj = rel_l2(p.object, g.out["object"])
    d_probe = rel_l2(p._probe, g.out["probe_corner"])

    floor = Oracle(state, fft_round_trip=True).reconstruct(**kw)
    f_err = float(np.max(np.abs(np.asarray(floor.error_iterations) - ref_err) / ref_err))
    f_obj = rel_l2(floor.object, g.out["object"])
    f_probe = rel_l2(floor.probe, g.out["probe_corner"])
    o64 = Oracle(state, "float64").reconstruct(**kw)
    print(f"\n{name}: gpu-vs-ref err {d_err:.2e} obj {d_obj:.2e} probe {d_probe:.2e} | "
          f"floor err {f_err:.2e} obj {f_obj:.2e} probe {f_probe:.2e} | "
          f"gpu-vs-fp64 obj {rel_l2(p.object, o64.object):.2e} "
          f"probe {rel_l2(p._probe, o64.probe):.2e} | "
          f"ref-vs-fp64 obj {rel_l2(g.out['object'], o64.object):.2e}")
    k = 5.0 if g.projection else 3.0
    tol_err = max(1e-5, k * f_err)
    tol_obj = max(1e-4, k * f_obj)
    tol_probe = max(1e-4, k * f_probe)
    if not g.projection and name not in FLOOR_BOUND:  # the parity bar as stated
        tol_err, tol_obj, tol_probe = 1e-5, 1e-4, 1e-4
    assert d_err <= tol_err
    if g.projection:
        # projection sets leave directions of the object the data do not constrain
        # to rounding: there it is enough that the GPU result lies at least as close
        # to the FP64 evaluation of the same model as the reference's own result
        assert d_obj <= tol_obj or (rel_l2(p.object, o64.object)
                                    <= rel_l2(g.out["object"], o64.object))
        assert d_probe <= tol_probe or (rel_l2(p._probe, o64.probe)
                                        <= rel_l2(g.out["probe_corner"], o64.probe))
    else:
        assert d_obj <= tol_obj
        assert d_probe <= tol_probe
    # position correction fixtures move the positions; the others leave them alone
    d_pos = float(np.max(np.abs(p._positions_px - g.out["positions_px"])))
    f_pos = float(np.max(np.abs(floor.positions_px - g.out["positions_px"])))
    print(f"{name}: positions gpu-vs-ref {d_pos:.2e} px, floor {f_pos:.2e} px")
    assert d_pos <= max(1e-4, k * f_pos)


@pytest.mark.parametrize("name", names())
def test_self_consistency_errors_match_reference(cuda, name):
    """Per-position errors of the reference's final state (A19): float64 values
    within 1e-5 relative of the reference (its own rounding floor is ~4e-7)."""
    g = Golden(name)
    p = g.build(device="gpu")
    p._object = np.array(g.out["object"], copy=True)
    p._probe = np.array(g.out["probe_corner"], copy=True)
    p._positions_px = np.array(g.out["positions_px"], copy=True)
    e = p._return_self_consistency_errors(
        max_batch_size=g.meta["reconstruct"].get("max_batch_size"))
    ref = g.out["self_consistency_errors"]
    assert e.dtype == np.float64 and e.shape == ref.shape
    rel = np.abs(e - ref) / ref
    print(f"\n{name}: self-consistency max rel {rel.max():.2e} mean {rel.mean():.2e}")
    assert rel.max() <= 1e-5


def test_storage_cpu_matches_gpu(cuda):
    g = Golden("ss_gd_potential")
    a = g.build(device="gpu", storage="gpu")
    b = g.build(device="gpu", storage="cpu")
    a.reconstruct(progress_bar=False, **g.meta["reconstruct"])
    b.reconstruct(progress_bar=False, **g.meta["reconstruct"])
    np.testing.assert_array_equal(a.object, b.object)
    np.testing.assert_array_equal(a._probe, b._probe)
    assert a.error_iterations == b.error_iterations


def test_storage_cpu_page_locked_matches_gpu(cuda):
    """Host amplitudes in page-locked memory, gathered to the device one batch
    ahead: the same result bit for bit."""
    torch = cuda
    from py4dstem_gb300 import engine

    g = Golden("ss_gd_potential")
    a = g.build(device="gpu", storage="gpu")
    b = g.build(device="gpu", storage="cpu")
    b._amplitudes = torch.from_numpy(np.ascontiguousarray(b._amplitudes)).pin_memory().numpy()
    assert engine.mapped_host_address(b._amplitudes) is not None
    assert engine.mapped_host_address(np.ones(16, np.float32)) is None  # pageable
    a.reconstruct(progress_bar=False, **g.meta["reconstruct"])
    b.reconstruct(progress_bar=False, **g.meta["reconstruct"])
    np.testing.assert_array_equal(a.object, b.object)
    np.testing.assert_array_equal(a._probe, b._probe)
    assert a.error_iterations == b.error_iterations


def test_continue_and_reset_semantics(cuda):
    g = Golden("ss_gd_potential")
    rec = dict(g.meta["reconstruct"])
    n = rec.pop("num_iter")
    a = g.build()
    a.reconstruct(num_iter=n, progress_bar=False, **rec)
    b = g.build()
    b.reconstruct(num_iter=2, progress_bar=False, **rec)
    b.reconstruct(num_iter=n - 2, progress_bar=False, reset=True, **rec)
    assert len(b.error_iterations) == n - 2
    c = g.build()
    c.reconstruct(num_iter=n, progress_bar=False, **rec)
    c.reconstruct(num_iter=1, progress_bar=False, **rec)  # continues
    assert len(c.error_iterations) == n + 1
    np.testing.assert_array_equal(a.error_iterations, c.error_iterations[:n])



@pytest.mark.parametrize("name", ["ss_gd_det128", "ms_gd_T3", "mixed_gd_M3", "ss_ap"])
def test_graph_replay_matches_eager(cuda, name):
    """Iterations replayed from one captured CUDA graph give the same bits as the
    same iterations issued kernel by kernel."""
    g = Golden(name)
    out = []
    for graph in (False, True):
        p = g.build()
        p._graph_iterations = graph
        p.reconstruct(**g.rec_kwargs())
        out.append((np.asarray(p._object), np.asarray(p._probe), list(p.error_iterations)))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


def test_save_read_continue(cuda, tmp_path):
    """A reconstruction saved, read back and preprocessed again continues from
    the saved object and probe."""
    import py4dstem_gb300 as pg

    g = Golden("ss_gd_det128")
    p = g.build()
    kw = g.rec_kwargs()
    kw["num_iter"] = 2
    p.reconstruct(**kw)
    p.set_save_defaults(save_datacube=True)
    p.save(tmp_path / "r.npz")
    q = pg.read(tmp_path / "r.npz")
    np.testing.assert_array_equal(q.object, p.object)
    np.testing.assert_array_equal(q.probe, p.probe)
    q.preprocess(**g.meta["preprocess"])
    np.testing.assert_array_equal(q._object, p._object)
    q.reconstruct(**dict(kw, num_iter=1))
    assert np.isfinite(q.error) and q.error < p.error_iterations[0]


def test_repeated_calls_reuse_state_and_match(cuda):
    """Consecutive reconstruct() calls with the same settings reuse the device
    state and the captured iteration graph, with the same bits as calls that
    build a new state each time; a change of settings builds a new state."""
    g = Golden("ss_gd_det128")
    kw = g.rec_kwargs()
    n = kw.pop("num_iter")
    b = g.build()
    c = g.build()
    states = set()
    for _ in range(n):
        b.reconstruct(num_iter=1, **kw)
        states.add(id(b._device_state))
        c.__dict__["_state_cache"] = None
        c.reconstruct(num_iter=1, **kw)
    assert len(states) == 1
    assert b.error_iterations == c.error_iterations
    np.testing.assert_array_equal(b.object, c.object)
    np.testing.assert_array_equal(b.probe, c.probe)
    st = b._device_state
    b.reconstruct(num_iter=1, **dict(kw, step_size=0.25))
    assert b._device_state is not st


@pytest.mark.parametrize("cls_modes", [1, 2])
def test_position_correction_128_grouped_and_block_wide(cuda, cls_modes):
    """Gradient descent with position correction at a 128^2 detector (the
    grouped kernels keep the far fields and correct the positions), against the
    oracle on the same preprocessed state and against the block-wide schedule."""
    from oracle.ptycho_np import Oracle
    from py4dstem_gb300 import _native

    lib = _native.lib()
    g = Golden("ss_gd_det128")
    extra = dict(fix_positions=False, fix_positions_com=False, positions_step_size=0.5,
                 max_position_update_distance=0.1, max_position_total_distance=0.3)
    if cls_modes > 1:
        g.meta = dict(g.meta, cls="mixed", ctor=dict(g.meta["ctor"], num_probes=cls_modes))
    kw = dict(g.rec_kwargs(), **extra)
    out = {}
    try:
        for schedule in (0, 1):
            lib.ptycho_set_kernel_schedule(128, schedule)
            p = g.build()
            if schedule == 0:
                state = g.state(p)
            p.reconstruct(progress_bar=False, **kw)
            out[schedule] = (np.asarray(p._object), np.asarray(p._probe),
                             np.asarray(p.error_iterations), np.array(p._positions_px))
    finally:
        lib.ptycho_set_kernel_schedule(128, 0)
    okw = dict(g.oracle_kwargs(), **extra)
    o = Oracle(state).reconstruct(**okw)
    obj, probe, err, pos = out[0]
    d_err = float(np.max(np.abs(err - o.error_iterations) / np.abs(o.error_iterations)))
    print(f"\ngrouped vs oracle: err {d_err:.2e} obj {rel_l2(obj, o.object):.2e} "
          f"probe {rel_l2(probe, o.probe):.2e} "
          f"pos {float(np.max(np.abs(pos - o.positions_px))):.2e} px")
    assert d_err < 2e-5
    assert rel_l2(obj, o.object) < 1e-4
    assert rel_l2(probe, o.probe) < 1e-4
    assert float(np.max(np.abs(pos - o.positions_px))) < 1e-3
    assert rel_l2(obj, out[1][0]) < 1e-5
    assert float(np.max(np.abs(pos - out[1][3]))) < 1e-3
