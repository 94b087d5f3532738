"""The C-ABI library: builds, loads, exports every declared symbol, and rejects bad
arguments on the host (no GPU call is made by these tests)."""

import ctypes
import os
import re

import pytest

from py4dstem_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ptycho_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ptycho_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    return _native.lib()


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(_native.EXPORTED_SYMBOLS)


def test_abi_version(lib):
    assert lib.ptycho_abi_version() == 5


@pytest.mark.parametrize("n,ok", [(32, 1), (48, 1), (64, 1), (96, 1), (128, 1), (80, 0),
                                  (256, 1), (100, 0), (512, 0)])
def test_roi_supported(lib, n, ok):
    assert lib.ptycho_roi_supported(n, n) == ok
    assert lib.ptycho_roi_supported(n, n * 2) == 0


def test_non_square_roi_supported(lib):
    assert lib.ptycho_roi_supported(96, 128) == 1
    assert lib.ptycho_roi_supported(128, 96) == 1
    assert lib.ptycho_roi_supported(64, 128) == 0


def geometry(roi=64, obj=128, T=1, M=1, potential=0):
    return _native.Geometry(roi, roi, obj, obj, T, M, potential, 0)


def test_workspace_size_grows_with_batch(lib):
    g = geometry()
    w1 = lib.ptycho_workspace_bytes(ctypes.byref(g), 1)
    w64 = lib.ptycho_workspace_bytes(ctypes.byref(g), 64)
    assert 0 < w1 < w64
    # per-position staging: object term c64 + |P|^2 + probe term c64 + |O|^2 + F c64 = 32 B/px
    assert w64 - w1 >= 63 * 64 * 64 * 32
    assert lib.ptycho_workspace_bytes(None, 4) == 0
    assert lib.ptycho_workspace_bytes(ctypes.byref(g), 0) == 0


def _gd(lib, g, ws=None, wsb=0, batch=4):
    dummy = ctypes.c_void_p(0x1000)
    return lib.ptycho_gd_batch(ctypes.byref(g) if g is not None else None, dummy, dummy, dummy,
                               None, dummy, None, batch, 0.5, 1.0, 0, None, None, dummy,
                               ws, wsb, None)


def test_rejects_null_geometry(lib):
    assert _gd(lib, None) == 1
    assert b"geometry" in lib.ptycho_last_error()


def test_rejects_unsupported_roi(lib):
    assert _gd(lib, geometry(roi=80)) == 2
    assert b"80x80" in lib.ptycho_last_error()


@pytest.mark.parametrize("T,M,flags,ok", [
    (1, 1, 0, True), (2, 1, 0, True), (1, 2, 0, True), (2, 2, 0, True),
    (1, 1, "FLAG_MIXED_STATE", True), (1, 1, "FLAG_KEEP_FARFIELD", False)])
def test_staged_roi_models(lib, T, M, flags, ok):
    """256 x 256 runs every gradient-descent model on the staged kernels; kept far
    fields (position correction) are refused on the host with the reason."""
    g = geometry(roi=256, obj=320, T=T, M=M)
    g.flags = getattr(_native, flags) if flags else 0
    status = lib.ptycho_geometry_supported(ctypes.byref(g))
    if ok:
        assert status == 0
        assert _gd(lib, g) == 3  # the geometry passed; the null workspace did not
    else:
        assert status == 2
        assert b"PTYCHO_FLAG_KEEP_FARFIELD" in lib.ptycho_last_error()
        assert _gd(lib, g) == 2


@pytest.mark.parametrize("det,status", [((0, 0), 0), ((48, 48), 0), ((96, 128), 0),
                                        ((0, 48), 1), ((1, 64), 1), ((-4, 64), 1),
                                        ((8192, 64), 2)])
def test_detector_shape_checks(lib, det, status):
    """The detector shape (resampled far field) is validated on the host."""
    g = geometry(roi=64, obj=128)
    g.detector_x, g.detector_y = det
    assert lib.ptycho_geometry_supported(ctypes.byref(g)) == status
    assert (lib.ptycho_workspace_bytes(ctypes.byref(g), 4) > 0) == (status == 0)


def test_resampled_workspace_holds_detector_far_fields(lib):
    g = geometry(roi=64, obj=128, M=2)
    base = lib.ptycho_workspace_bytes(ctypes.byref(g), 8)
    g.detector_x, g.detector_y = 96, 96
    # + B M Ax Ay c64 detector far fields and the error partials
    assert lib.ptycho_workspace_bytes(ctypes.byref(g), 8) >= base + 8 * 2 * 96 * 96 * 8
    g.flags = _native.FLAG_KEEP_FARFIELD
    assert lib.ptycho_geometry_supported(ctypes.byref(g)) == 2


def test_geometry_supported_matches_the_batch_checks(lib):
    assert lib.ptycho_geometry_supported(None) == 1
    assert lib.ptycho_geometry_supported(ctypes.byref(geometry(roi=80))) == 2
    assert lib.ptycho_geometry_supported(ctypes.byref(geometry(roi=64, obj=48))) == 2
    assert lib.ptycho_geometry_supported(ctypes.byref(geometry(T=2, M=2))) == 0


def test_staged_roi_refused_by_the_engine():
    """The engine raises NotImplementedError for options the 256 x 256 kernels
    do not run, before any device work."""
    import numpy as np

    from py4dstem_gb300 import engine

    with pytest.raises(NotImplementedError, match="PTYCHO_FLAG_KEEP_FARFIELD"):
        engine.create_state(roi_shape=(256, 256), object_array=np.ones((320, 320), np.complex64),
                            probe_array=np.ones((256, 256), np.complex64),
                            amplitudes=np.ones((4, 256, 256), np.float32),
                            positions_px=np.zeros((4, 2), np.float32), num_slices=1,
                            num_probes=1, potential=False, max_batch=4,
                            positions_initial=np.zeros((4, 2), np.float32))
    with pytest.raises(NotImplementedError, match="projection sets"):
        engine.create_state(roi_shape=(256, 256), object_array=np.ones((320, 320), np.complex64),
                            probe_array=np.ones((256, 256), np.complex64),
                            amplitudes=np.ones((4, 256, 256), np.float32),
                            positions_px=np.zeros((4, 2), np.float32), num_slices=1,
                            num_probes=1, potential=False, max_batch=4, projection=True)


def test_rejects_object_smaller_than_roi(lib):
    assert _gd(lib, geometry(roi=64, obj=48)) == 2


def test_mixed_multislice_geometry(lib):
    """Mixed-state multislice geometries are accepted (the calls get as far as the
    workspace check here); the workspace holds every slice's probe per mode."""
    g = geometry(T=2, M=2)
    assert _gd(lib, g) == 3  # null workspace: the geometry itself was accepted
    need = lib.ptycho_workspace_bytes(ctypes.byref(g), 4)
    # + T B M N c64 stash + B M N c64 far fields over the single-probe multislice
    base = lib.ptycho_workspace_bytes(ctypes.byref(geometry(T=2, M=1)), 4)
    assert need >= base + (2 * 4 * 2 + 4 * 2) * 64 * 64 * 8 - 4 * 64 * 64 * 8


def test_rejects_bad_batch_and_workspace(lib):
    g = geometry()
    assert _gd(lib, g, batch=0) == 1
    assert _gd(lib, g, ws=None) == 3
    assert _gd(lib, g, ws=ctypes.c_void_p(0x1001), wsb=1 << 30) == 3  # misaligned
    assert _gd(lib, g, ws=ctypes.c_void_p(0x1000), wsb=16) == 3       # too small
    assert b"smaller" in lib.ptycho_last_error()


def test_rejects_unknown_flags(lib):
    g = geometry()
    g.flags = 16
    assert _gd(lib, g) == 1
    assert b"flags" in lib.ptycho_last_error()


def _pc(lib, g, ws=ctypes.c_void_p(0x1000), wsb=1 << 40, initial=ctypes.c_void_p(0x1000)):
    dummy = ctypes.c_void_p(0x1000)
    return lib.ptycho_position_correction(ctypes.byref(g), dummy, None, None, dummy, None,
                                          dummy, initial, None, 4, 0.5, -1.0, -1.0, ws, wsb,
                                          None)


def test_position_correction_argument_checks(lib):
    g = geometry()
    assert _pc(lib, g) == 1  # far fields were not kept
    assert b"KEEP_FARFIELD" in lib.ptycho_last_error()
    g.flags = _native.FLAG_KEEP_FARFIELD
    assert _pc(lib, g, initial=None) == 1
    assert b"positions_initial" in lib.ptycho_last_error()
    assert _pc(lib, g, ws=None) == 3
    g = geometry(T=3)
    g.flags = _native.FLAG_KEEP_FARFIELD
    assert _pc(lib, g) == 1
    assert b"propagators" in lib.ptycho_last_error()


def test_keep_farfield_workspace(lib):
    g = geometry(T=3)
    base = lib.ptycho_workspace_bytes(ctypes.byref(g), 8)
    g.flags = _native.FLAG_KEEP_FARFIELD
    # multislice keeps one far field (c64) per position only when asked to
    assert lib.ptycho_workspace_bytes(ctypes.byref(g), 8) >= base + 8 * 64 * 64 * 8


def test_self_consistency_argument_checks(lib):
    dummy = ctypes.c_void_p(0x1000)
    g = geometry()
    st = lib.ptycho_self_consistency_errors(ctypes.byref(g), dummy, dummy, dummy, None, dummy,
                                            None, 4, None, None, dummy, 1 << 40, None)
    assert st == 1 and b"errors" in lib.ptycho_last_error()
    g = geometry(T=3)
    st = lib.ptycho_self_consistency_errors(ctypes.byref(g), dummy, dummy, dummy, None, dummy,
                                            None, 4, None, dummy, dummy, 1 << 40, None)
    assert st == 1 and b"propagators" in lib.ptycho_last_error()


def _noalloc(lib, g, batch):
    dummy = ctypes.c_void_p(0x1000)
    return lib.ptycho_gd_batch_noalloc(ctypes.byref(g), dummy, dummy, dummy, None, dummy, None,
                                       batch, 0.5, 1.0, 0, None, None, dummy, None)


def test_noalloc_refuses_batches_beyond_its_scratch(lib):
    """The no-allocation entry point refuses a batch whose scratch exceeds its
    fixed 32 MiB array, before any GPU work."""
    g = _native.Geometry(128, 128, 512, 512, 1, 1, 0, 0)
    assert lib.ptycho_workspace_bytes(ctypes.byref(g), 4096) > (32 << 20)
    assert _noalloc(lib, g, 4096) == 3
    assert b"no-allocation scratch" in lib.ptycho_last_error()


@pytest.mark.parametrize("flag", ["FLAG_SPECTRUM_READY", "FLAG_PREPARE_SPECTRUM",
                                  "FLAG_KEEP_FARFIELD"])
def test_noalloc_refuses_batch_chaining_flags(lib, flag):
    """Flags that pass data from one call to the next through the scratch are
    refused: every no-allocation call shares that scratch."""
    g = geometry()
    g.flags = getattr(_native, flag)
    assert _noalloc(lib, g, 4) == 1
    assert b"ptycho_gd_batch_noalloc does not take" in lib.ptycho_last_error()


def test_read_error_argument_checks(lib):
    value = ctypes.c_float(0.0)
    assert lib.ptycho_read_error(None, ctypes.byref(value), None) == 1
    assert lib.ptycho_read_error(ctypes.c_void_p(0x1000), None, None) == 1
    assert b"non-null" in lib.ptycho_last_error()


def test_nonfinite_positions_rejected_on_the_host():
    """NaN or infinite scan positions are refused before any device work."""
    import numpy as np

    from py4dstem_gb300 import engine

    pos = np.zeros((4, 2), np.float32)
    pos[1, 0] = np.nan
    with pytest.raises(ValueError, match="NaN or infinite"):
        engine.create_state(roi_shape=(64, 64), object_array=np.ones((96, 96), np.complex64),
                            probe_array=np.ones((64, 64), np.complex64),
                            amplitudes=np.ones((4, 64, 64), np.float32), positions_px=pos,
                            num_slices=1, num_probes=1, potential=False, max_batch=4)


def test_gather_patterns_argument_checks(lib):
    """The batch gather refuses bad counts and null pointers before any device
    work; an empty gather is a no-op."""
    p = ctypes.c_void_p(0x1000)
    assert lib.ptycho_gather_patterns(p, 4, 16, None, 0, p, None) == 0
    assert lib.ptycho_gather_patterns(p, 4, 16, None, -1, p, None) == 1
    assert lib.ptycho_gather_patterns(p, 4, 0, None, 2, p, None) == 1
    assert lib.ptycho_gather_patterns(None, 4, 16, None, 2, p, None) == 1
    assert b"null pointer" in lib.ptycho_last_error()
    assert lib.ptycho_gather_patterns(p, 4, 16, None, 2, None, None) == 1
    # without a row list the first num_out patterns are taken: there must be as many
    assert lib.ptycho_gather_patterns(p, 4, 16, None, 5, p, None) == 1
    assert b"5 rows requested of 4 patterns" in lib.ptycho_last_error()


def test_kernel_schedule_argument_checks(lib):
    """Schedules 0-3 are taken (the previous one returned), others refused; the
    setting is process-wide and is put back."""
    prev = lib.ptycho_set_kernel_schedule(128, 3)
    try:
        assert lib.ptycho_set_kernel_schedule(128, 1) == 3
        assert lib.ptycho_set_kernel_schedule(128, 0) == 1
        assert lib.ptycho_set_kernel_schedule(128, 4) == -1  # -PTYCHO_ERR_INVALID_ARGUMENT
        assert b"schedule must be 0, 1, 2 or 3" in lib.ptycho_last_error()
        assert lib.ptycho_set_kernel_schedule(128, -1) == -1
        assert lib.ptycho_set_kernel_schedule(128, 2) == 0  # unchanged by the refusals
    finally:
        lib.ptycho_set_kernel_schedule(128, prev)
