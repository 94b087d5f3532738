"""Failure detection without a GPU fault: non-finite inputs make the batch error
sum NaN on the device, and the per-iteration read-back (ptycho_read_error)
reports PTYCHO_ERR_NONFINITE. Every failure here is made on the host (a NaN or
infinite value written into an input array); no kernel is made to fault, trap
or hang, and each test checks that the GPU context still runs a clean batch
afterwards."""

import ctypes

import numpy as np
import pytest

from gpu_helpers import make_state
from py4dstem_gb300 import _native

pytestmark = pytest.mark.gpu

NONFINITE = 5


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _batch_status(torch, st, poison=None):
    """One gradient-descent batch over all positions of `st` through the C ABI,
    with `poison(arrays)` applied to the host inputs first; returns the status
    of ptycho_read_error and the error value."""
    lib = _native.lib()
    dev = torch.device("cuda")
    arrays = dict(object=np.ascontiguousarray(st.object, dtype=np.complex64).copy(),
                  probe=np.ascontiguousarray(st.probe, dtype=np.complex64).copy(),
                  amplitudes=np.ascontiguousarray(st.amplitudes).copy(),
                  positions=np.ascontiguousarray(st.positions_px).copy())
    if poison is not None:
        poison(arrays)
    t = {k: torch.from_numpy(v).to(dev) for k, v in arrays.items()}
    J = st.amplitudes.shape[0]
    S = st.amplitudes.shape[-1]
    P = st.object.shape[-1]
    g = _native.Geometry(S, S, P, P, 1, 1, 0, 0)
    nbytes = lib.ptycho_workspace_bytes(ctypes.byref(g), J)
    ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
    err = torch.zeros(1, dtype=torch.float32, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    status = lib.ptycho_gd_batch(ctypes.byref(g), _ptr(t["object"]), _ptr(t["probe"]),
                                 _ptr(t["amplitudes"]), None, _ptr(t["positions"]), None, J,
                                 0.5, 1.0, 0, None, None, _ptr(err),
                                 ctypes.c_void_p((ws.data_ptr() + 255) & ~255), nbytes, stream)
    assert status == 0, lib.ptycho_last_error()
    value = ctypes.c_float(0.0)
    status = lib.ptycho_read_error(_ptr(err), ctypes.byref(value), stream)
    return status, value.value, t


def _nan_amplitude(a):
    a["amplitudes"][3, 5, 7] = np.nan


def _inf_amplitude(a):
    a["amplitudes"][0, 0, 0] = np.inf


def _nan_probe(a):
    a["probe"][10, 11] = np.complex64(np.nan)


def _nan_object(a):
    a["object"][:] = np.complex64(np.nan)


def _nan_position(a):
    a["positions"][2, 0] = np.nan


def _inf_position(a):
    a["positions"][4, 1] = -np.inf


@pytest.mark.parametrize("poison", [_nan_amplitude, _inf_amplitude, _nan_probe, _nan_object,
                                    _nan_position, _inf_position],
                         ids=lambda f: f.__name__.lstrip("_"))
def test_nonfinite_input_is_reported(cuda, poison):
    st = make_state(S=64, J=9, seed=41)
    status, value, _ = _batch_status(cuda, st, poison)
    assert status == NONFINITE, (status, value)
    assert not np.isfinite(value)
    assert b"NaN or infinite" in _native.lib().ptycho_last_error()
    # the context is intact: a clean batch runs and reads back a finite error
    status, value, t = _batch_status(cuda, st)
    assert status == 0 and np.isfinite(value) and value > 0
    assert bool(cuda.isfinite(t["object"]).all())


def test_nonfinite_position_keeps_indices_inside_the_object(cuda):
    """A NaN position is read as 0 for its patch indices: the batch completes,
    the other positions' updates stay finite, and only the error reports it."""
    st = make_state(S=64, J=9, seed=42)
    status, _, t = _batch_status(cuda, st, _nan_position)
    assert status == NONFINITE
    assert bool(cuda.isfinite(t["object"]).all())
    assert bool(cuda.isfinite(t["probe"]).all())


def test_reconstruct_raises_on_nan_amplitudes_and_recovers(cuda):
    """Through the public API: NaN amplitudes end reconstruct() with a
    RuntimeError (status PTYCHO_ERR_NONFINITE); a clean reconstruction on the
    same GPU afterwards succeeds."""
    from golden_io import Golden

    g = Golden("ss_gd_det128")
    p = g.build(device="gpu", storage="cpu")
    amps = np.array(p._amplitudes, copy=True)
    amps[1, 2, 3] = np.nan
    p._amplitudes = amps
    with pytest.raises(_native.PtychoError) as info:
        p.reconstruct(**g.rec_kwargs())
    assert info.value.status == NONFINITE
    q = g.build(device="gpu")
    q.reconstruct(**g.rec_kwargs())
    assert np.all(np.isfinite(q.error_iterations))
