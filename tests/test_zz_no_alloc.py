"""ptycho_gd_batch_noalloc: the gradient-descent batch for callers that cannot
allocate device memory, so they cannot hand the library a workspace. Examples
are an acquisition loop whose device-memory budget is fixed when the microscope
session starts, and a host application whose own allocator owns the GPU.

Each test goes through the C ABI and compares the entry point with
ptycho_gd_batch on a caller workspace. Both run the same kernels with the same
scratch layout (the layout does not depend on the buffer's size), so the
results must be bit-identical. The cases:
  - single-slice, multislice and mixed-state geometries, each on two
    consecutive batches;
  - a second pair of calls on the scratch the first pair left behind;
  - the largest batch whose scratch fits the fixed array.
The CPU tests in test_native_abi.py cover the refusals: batches beyond the
array and the batch-chaining flags.

The file builds its own inputs and depends on no other test. It passes alone
in a fresh process and after the rest of the suite. Its name sorts last, so a
run that stops at the first failure has run every other test before this one.
"""

import ctypes

import numpy as np
import pytest

from gpu_helpers import make_state
from py4dstem_gb300 import _native

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 32 << 20  # the fixed no-allocation scratch of the library


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _geometry(st):
    S = st.amplitudes.shape[-1]
    P = st.object.shape[-1]
    return _native.Geometry(S, S, P, P, st.num_slices, st.num_probes, 0,
                            1 if st.mixed else 0)


def _run_batches(torch, lib, st, batch, calls, noalloc):
    """`calls` consecutive batches of `batch` positions; returns object, probe,
    error sum (all as host arrays)."""
    dev = torch.device("cuda")
    g = _geometry(st)
    obj = torch.from_numpy(np.ascontiguousarray(st.object, dtype=np.complex64)).to(dev)
    probe = torch.from_numpy(np.ascontiguousarray(st.probe, dtype=np.complex64)).to(dev)
    amps = torch.from_numpy(np.ascontiguousarray(st.amplitudes)).to(dev)
    pos = torch.from_numpy(np.ascontiguousarray(st.positions_px)).to(dev)
    props = (torch.from_numpy(np.ascontiguousarray(st.propagators, dtype=np.complex64)).to(dev)
             if st.num_slices > 1 else None)
    rows = torch.arange(st.amplitudes.shape[0], dtype=torch.int32, device=dev)
    err = torch.zeros(1, dtype=torch.float32, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if not noalloc:
        nbytes = lib.ptycho_workspace_bytes(ctypes.byref(g), batch)
        ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
        ws_ptr = ctypes.c_void_p((ws.data_ptr() + 255) & ~255)
    for k in range(calls):
        rows_ptr = ctypes.c_void_p(rows.data_ptr() + 4 * k * batch)
        common = (ctypes.byref(g), _ptr(obj), _ptr(probe), _ptr(amps), rows_ptr, _ptr(pos),
                  rows_ptr, batch, 0.5, 1.0, 0, None, _ptr(props), _ptr(err))
        if noalloc:
            status = lib.ptycho_gd_batch_noalloc(*common, stream)
        else:
            status = lib.ptycho_gd_batch(*common, ws_ptr, nbytes, stream)
        assert status == 0, lib.ptycho_last_error()
    torch.cuda.synchronize()
    return obj.cpu().numpy(), probe.cpu().numpy(), err.cpu().numpy()


def _assert_same(a, b):
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


CASES = {
    "single": dict(S=64, J=24, seed=31),
    "multislice": dict(S=64, J=16, slices=3, seed=32),
    "mixed": dict(S=64, J=16, modes=3, seed=33),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_noalloc_matches_workspace_entry_point(cuda, case):
    lib = _native.lib()
    st = make_state(**CASES[case])
    batch = st.amplitudes.shape[0] // 2
    ref = _run_batches(cuda, lib, st, batch, 2, noalloc=False)
    _assert_same(_run_batches(cuda, lib, st, batch, 2, noalloc=True), ref)
    # the same two calls again, on the scratch the previous calls left behind
    _assert_same(_run_batches(cuda, lib, st, batch, 2, noalloc=True), ref)


def test_noalloc_largest_batch_that_fits(cuda):
    """The largest batch whose scratch fits the fixed array runs and matches the
    workspace entry point; one position more is refused before any GPU work."""
    lib = _native.lib()
    S = 64
    P = 160
    g = _native.Geometry(S, S, P, P, 1, 1, 0, 0)
    lo, hi = 1, 4096
    while lo < hi:  # largest batch with workspace bytes <= the scratch
        mid = (lo + hi + 1) // 2
        if lib.ptycho_workspace_bytes(ctypes.byref(g), mid) <= SCRATCH_BYTES:
            lo = mid
        else:
            hi = mid - 1
    best = lo
    assert lib.ptycho_workspace_bytes(ctypes.byref(g), best + 1) > SCRATCH_BYTES
    st = make_state(S=S, J=best, seed=34, obj_px=P)
    assert st.object.shape[-1] == P
    ref = _run_batches(cuda, lib, st, best, 1, noalloc=False)
    _assert_same(_run_batches(cuda, lib, st, best, 1, noalloc=True), ref)
    dummy = ctypes.c_void_p(0x1000)
    status = lib.ptycho_gd_batch_noalloc(ctypes.byref(g), dummy, dummy, dummy, None, dummy, None,
                                         best + 1, 0.5, 1.0, 0, None, None, dummy, None)
    assert status == 3
    assert b"no-allocation scratch" in lib.ptycho_last_error()
