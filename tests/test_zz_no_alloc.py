"""ptycho_gd_batch_noalloc: the gradient-descent batch for callers that cannot
allocate device memory (for example an acquisition loop whose device-memory
budget is fixed when the session starts, or a host application whose own
allocator owns the GPU), so they cannot hand the library a workspace.

Checked through the C ABI against ptycho_gd_batch with a caller workspace, on two
consecutive batches (the second call reuses the shared scratch the first one
left behind). Also checked: a batch larger than the fixed scratch is refused
before any GPU work.

This file is collected last on purpose; it builds its own inputs, so it passes
alone in a fresh process and after the rest of the suite.
"""

import ctypes

import numpy as np
import pytest

from gpu_helpers import make_state, rel
from py4dstem_gb300 import _native

pytestmark = pytest.mark.gpu

TOL = 2e-5  # the kernel-parity tolerance of tests/test_gpu_kernels.py


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _run_two_batches(torch, lib, st, batch, noalloc):
    dev = torch.device("cuda")
    J = st.amplitudes.shape[0]
    S = st.amplitudes.shape[-1]
    P = st.object.shape[-1]
    g = _native.Geometry(S, S, P, P, 1, 1, 0, 0)
    obj = torch.from_numpy(np.ascontiguousarray(st.object, dtype=np.complex64)).to(dev)
    probe = torch.from_numpy(np.ascontiguousarray(st.probe, dtype=np.complex64)).to(dev)
    amps = torch.from_numpy(np.ascontiguousarray(st.amplitudes)).to(dev)
    pos = torch.from_numpy(np.ascontiguousarray(st.positions_px)).to(dev)
    rows = torch.arange(J, dtype=torch.int32, device=dev)
    err = torch.zeros(1, dtype=torch.float32, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ws = None
    if not noalloc:
        nbytes = lib.ptycho_workspace_bytes(ctypes.byref(g), batch)
        ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
        ws_ptr = ctypes.c_void_p((ws.data_ptr() + 255) & ~255)
    for start in range(0, 2 * batch, batch):
        rows_ptr = ctypes.c_void_p(rows.data_ptr() + 4 * start)
        common = (ctypes.byref(g), _ptr(obj), _ptr(probe), _ptr(amps), rows_ptr, _ptr(pos),
                  rows_ptr, batch, 0.5, 1.0, 0, None, None, _ptr(err))
        if noalloc:
            status = lib.ptycho_gd_batch_noalloc(*common, stream)
        else:
            status = lib.ptycho_gd_batch(*common, ws_ptr, nbytes, stream)
        assert status == 0, lib.ptycho_last_error()
    torch.cuda.synchronize()
    return obj.cpu().numpy(), probe.cpu().numpy(), float(err.item())


def test_noalloc_matches_workspace_entry_point(cuda):
    lib = _native.lib()
    st = make_state(S=64, J=24, seed=31)
    ref_obj, ref_probe, ref_err = _run_two_batches(cuda, lib, st, 12, noalloc=False)
    obj, probe, err = _run_two_batches(cuda, lib, st, 12, noalloc=True)
    assert rel(obj, ref_obj) < TOL
    assert rel(probe, ref_probe) < TOL
    assert abs(err - ref_err) <= TOL * abs(ref_err)
    # a second pair of calls on the now-used scratch gives the same answer
    obj2, probe2, err2 = _run_two_batches(cuda, lib, st, 12, noalloc=True)
    assert rel(obj2, ref_obj) < TOL and rel(probe2, ref_probe) < TOL
    assert abs(err2 - ref_err) <= TOL * abs(ref_err)


def test_noalloc_refuses_batches_beyond_its_scratch():
    lib = _native.lib()
    g = _native.Geometry(128, 128, 512, 512, 1, 1, 0, 0)
    dummy = ctypes.c_void_p(0x1000)
    status = lib.ptycho_gd_batch_noalloc(ctypes.byref(g), dummy, dummy, dummy, None, dummy, None,
                                         4096, 0.5, 1.0, 0, None, None, dummy, None)
    assert status == 3
    assert b"no-allocation scratch" in lib.ptycho_last_error()
