"""Device state and the iteration driver of the GPU reconstruction.

The host keeps what the reference keeps on the host: the iteration and batch
loops, NumPy's global RNG for the position order (singleslice_ptychography.py:836-857)
and the error bookkeeping. Every array operation of an iteration is a call into
libptycho_gb300 on the current CUDA stream; torch is used only to own device
memory and to name the stream.

Per batch: ptycho_gd_batch / ptycho_projection_batch (forward, projection,
adjoint, deterministic scatter, object and probe update). Per iteration:
object constraints, probe centre-of-mass constraint and, for mixed states, the
probe orthogonalisation (Gram matrix on the GPU, the M x M eigendecomposition on
the host as numpy.linalg.eigh, mode mixing on the GPU).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _native
from .preprocess import generate_batches


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError(
            "py4dstem_gb300 reconstructs on a CUDA GPU only and none is available "
            "(there is no CPU fallback)")
    return torch


def _ptr(t) -> Optional[int]:
    return None if t is None else ctypes.c_void_p(t.data_ptr())


@dataclass
class DeviceState:
    """All device buffers of one reconstruction."""

    geometry: _native.Geometry
    object: object
    probe: object
    amplitudes: object            # device (J,Sx,Sy) f32, or None when streamed
    amplitudes_host: Optional[np.ndarray]
    positions: object             # device (J,2) f32
    order: object                 # device (J,) int32
    workspace: object
    workspace_bytes: int
    error_accum: object
    max_batch: int
    propagators: object = None
    det_mask: object = None
    fov_mask_inverse: object = None
    exit_waves: object = None
    exit_waves_valid: bool = False
    amp_mapped: Optional[int] = None  # device address of page-locked host amplitudes
    amp_ring: object = None       # (2, max_batch, det) device batch buffers, filled one
                                  # batch ahead from amp_mapped on the prefetch stream
    ring_ready: object = None     # gather-done events of the two ring slots
    ring_free: object = None      # last-reader-done events of the two ring slots
    prefetch_stream: object = None
    amp_stage: object = None      # device batch buffer when streaming from the host
    amp_pinned: object = None     # two pinned host batch buffers (double-buffered)
    amp_events: object = None     # copy-done events of the pinned buffers
    amp_turn: int = 0
    order_pinned: object = None   # two pinned host buffers for the per-iteration order
    order_events: object = None
    order_turn: int = 0
    gram: object = None
    probe_tmp: object = None
    coeffs: object = None
    positions_initial: object = None  # device (J,2) f32 when positions are corrected
    launches: int = 0
    extra: dict = field(default_factory=dict)


# The region of interest whose model runs as batch-wide staged kernels (a wave
# does not fit one block's shared memory): gradient descent only, as for a far
# field resampled to a detector of another shape.
STAGED_ROI = (256, 256)


def supported_roi(shape) -> bool:
    return bool(_native.lib().ptycho_roi_supported(int(shape[0]), int(shape[1])))


def make_geometry(roi_shape, object_shape, num_slices, num_probes, potential,
                  mixed_state=False, detector_shape=None) -> _native.Geometry:
    """detector_shape: the amplitudes' shape when it differs from roi_shape (the
    far field is then resampled between the two grids)."""
    g = _native.Geometry(int(roi_shape[0]), int(roi_shape[1]), int(object_shape[-2]),
                         int(object_shape[-1]), int(num_slices), int(num_probes),
                         1 if potential else 0,
                         _native.FLAG_MIXED_STATE if mixed_state else 0)
    if detector_shape is not None and tuple(detector_shape) != tuple(roi_shape):
        g.detector_x, g.detector_y = int(detector_shape[0]), int(detector_shape[1])
    return g


def create_state(*, roi_shape, object_array, probe_array, amplitudes, positions_px,
                 num_slices, num_probes, potential, max_batch, storage="gpu",
                 propagators=None, detector_mask=None, fov_mask_inverse=None,
                 projection=False, mixed_state=False, positions_initial=None) -> DeviceState:
    if not np.all(np.isfinite(np.asarray(positions_px))):
        raise ValueError("scan positions contain NaN or infinite values")
    lib = _native.lib()
    det_shape = tuple(int(v) for v in np.shape(amplitudes)[-2:])
    geom = make_geometry(roi_shape, object_array.shape, num_slices, num_probes, potential,
                         mixed_state or num_probes > 1, det_shape)
    resampled = det_shape != tuple(int(v) for v in roi_shape)
    if positions_initial is not None:
        geom.flags |= _native.FLAG_KEEP_FARFIELD
    if not lib.ptycho_roi_supported(geom.roi_x, geom.roi_y):
        raise NotImplementedError(
            f"no GPU kernel for a {geom.roi_x}x{geom.roi_y} region of interest "
            "(supported: square 32, 48, 64, 96, 128, 256 and 96 x 128, 128 x 96)")
    if lib.ptycho_geometry_supported(ctypes.byref(geom)) != _native.PTYCHO_OK:
        raise NotImplementedError(lib.ptycho_last_error().decode())
    if projection and ((geom.roi_x, geom.roi_y) == STAGED_ROI or resampled):
        raise NotImplementedError(
            f"projection sets are not available for a {geom.roi_x}x{geom.roi_y} region of "
            "interest or a far field resampled to the detector")
    torch = _torch()
    dev = torch.device("cuda", torch.cuda.current_device())
    ws_bytes = int(lib.ptycho_workspace_bytes(ctypes.byref(geom), int(max_batch)))
    if ws_bytes == 0:
        raise ValueError("invalid geometry for the workspace query")
    obj_np = np.ascontiguousarray(object_array)
    obj = torch.from_numpy(obj_np).to(dev)
    probe_np = np.ascontiguousarray(probe_array, dtype=np.complex64).reshape(
        (num_probes,) + tuple(roi_shape))
    probe = torch.from_numpy(probe_np).to(dev)
    amps_dev = None
    amps_host = None
    amp_stage = amp_pinned = None
    mapped = None
    if isinstance(amplitudes, torch.Tensor) and storage != "gpu":
        amplitudes = amplitudes.cpu().numpy()
    if isinstance(amplitudes, torch.Tensor):
        # device amplitudes (from the device preprocessing) are used in place
        amps_dev = amplitudes.to(device=dev, dtype=torch.float32).contiguous()
    elif storage == "gpu":
        amps_dev = torch.from_numpy(np.ascontiguousarray(amplitudes, dtype=np.float32)).to(dev)
    else:
        amps_host = np.ascontiguousarray(amplitudes, dtype=np.float32)
        mapped = mapped_host_address(amps_host)
        if mapped is None:
            amp_stage = torch.empty((max_batch,) + det_shape, dtype=torch.float32,
                                    device=dev)
            amp_pinned = [torch.empty((max_batch,) + det_shape, dtype=torch.float32,
                                      pin_memory=True) for _ in range(2)]
    pos = torch.from_numpy(np.ascontiguousarray(positions_px, dtype=np.float32)).to(dev)
    order = torch.arange(pos.shape[0], dtype=torch.int32, device=dev)
    ws = torch.empty(ws_bytes + 256, dtype=torch.uint8, device=dev)
    err = torch.zeros(1, dtype=torch.float32, device=dev)
    st = DeviceState(geometry=geom, object=obj, probe=probe, amplitudes=amps_dev,
                     amplitudes_host=amps_host, positions=pos, order=order, workspace=ws,
                     workspace_bytes=ws_bytes, error_accum=err, max_batch=int(max_batch),
                     amp_stage=amp_stage, amp_pinned=amp_pinned, amp_mapped=mapped)
    if mapped is not None:
        # page-locked host amplitudes: each batch's patterns are gathered into a
        # device slot one batch ahead, on a second stream, while the batch before
        # it computes (the link's transfer hidden behind the batch instead of
        # stalling the position kernels that would read the rows in place)
        st.amp_ring = torch.empty((2, int(max_batch)) + det_shape, dtype=torch.float32,
                                  device=dev)
        st.ring_ready = [torch.cuda.Event(), torch.cuda.Event()]
        st.ring_free = [torch.cuda.Event(), torch.cuda.Event()]
        st.prefetch_stream = torch.cuda.Stream(device=dev)
    if propagators is not None:
        st.propagators = torch.from_numpy(
            np.ascontiguousarray(propagators, dtype=np.complex64)).to(dev)
    if detector_mask is not None:
        st.det_mask = torch.from_numpy(
            np.ascontiguousarray(np.asarray(detector_mask), dtype=np.float32)).to(dev)
    if fov_mask_inverse is not None:
        st.fov_mask_inverse = torch.from_numpy(
            np.ascontiguousarray(fov_mask_inverse, dtype=np.uint8)).to(dev)
    if projection:
        J = pos.shape[0]
        st.exit_waves = torch.empty((J, num_probes) + tuple(roi_shape), dtype=torch.complex64,
                                    device=dev)
    if positions_initial is not None:
        st.positions_initial = torch.from_numpy(
            np.ascontiguousarray(positions_initial, dtype=np.float32)).to(dev)
    if num_probes > 1:
        st.gram = torch.empty((num_probes, num_probes), dtype=torch.complex64, device=dev)
        st.probe_tmp = torch.empty_like(probe)
        st.coeffs = torch.empty((num_probes, num_probes), dtype=torch.complex64, device=dev)
    return st


def refresh_state(st: DeviceState, *, object_array, probe_array, positions_px,
                  detector_mask=None, fov_mask_inverse=None, positions_initial=None) -> None:
    """Copy new values of the per-call inputs into an existing state's buffers
    (same shapes), so that kernels and captured graphs that hold its pointers run
    on them."""
    torch = _torch()
    if not np.all(np.isfinite(np.asarray(positions_px))):
        raise ValueError("scan positions contain NaN or infinite values")

    def put(dst, arr, dtype):
        src = torch.from_numpy(np.ascontiguousarray(arr, dtype=dtype).reshape(tuple(dst.shape)))
        dst.copy_(src)

    put(st.object, object_array, np.asarray(object_array).dtype)
    put(st.probe, probe_array, np.complex64)
    put(st.positions, positions_px, np.float32)
    if detector_mask is not None:
        put(st.det_mask, np.asarray(detector_mask), np.float32)
    if fov_mask_inverse is not None:
        put(st.fov_mask_inverse, fov_mask_inverse, np.uint8)
    if positions_initial is not None:
        put(st.positions_initial, positions_initial, np.float32)


def _ws_ptr(st: DeviceState):
    base = st.workspace.data_ptr()
    aligned = (base + 255) & ~255
    return ctypes.c_void_p(aligned)


def _stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def mapped_host_address(array: np.ndarray) -> Optional[int]:
    """Device address of a page-locked host array (the GPU reads it directly over
    the CPU-GPU link), or None when the array lives in pageable memory."""
    lib = _native.lib()
    if array.nbytes == 0:
        return None
    dev = ctypes.c_void_p()
    _native.check(lib.ptycho_mapped_host_pointer(ctypes.c_void_p(array.ctypes.data),
                                                  ctypes.c_size_t(array.nbytes),
                                                  ctypes.byref(dev)))
    return dev.value or None


def _batch_amplitudes(st: DeviceState, start: int, end: int, host_order: np.ndarray):
    """(amplitudes pointer, amplitude rows pointer) of one batch: the resident
    array indexed by the order rows; page-locked host amplitudes read in place by
    the kernels (indexed the same way); or this batch's patterns gathered on the
    host and copied over."""
    n = end - start
    rows_ptr = ctypes.c_void_p(st.order.data_ptr() + 4 * start)
    if st.amplitudes is not None:
        return _ptr(st.amplitudes), rows_ptr
    if st.amp_mapped is not None:
        return ctypes.c_void_p(st.amp_mapped), rows_ptr
    else:
        # storage on the host: gather this batch's patterns and copy them over,
        # like the reference's per-batch copy_to_device
        torch = _torch()
        if st.amp_events is None:
            st.amp_events = [torch.cuda.Event(), torch.cuda.Event()]
        k = st.amp_turn
        st.amp_turn ^= 1
        st.amp_events[k].synchronize()  # the previous copy out of this buffer is done
        pinned = st.amp_pinned[k]
        idx = host_order[start:end]
        np.take(st.amplitudes_host, idx, axis=0, out=pinned.numpy()[:n])
        st.amp_stage[:n].copy_(pinned[:n], non_blocking=True)
        st.amp_events[k].record()
        return _ptr(st.amp_stage), None


def _gather_batch(st: DeviceState, slot: int, start: int, end: int) -> None:
    """On the prefetch stream, once ring slot `slot` is free: gather the patterns
    of order[start:end] from the page-locked host amplitudes into the slot."""
    lib = _native.lib()
    ps = st.prefetch_stream
    ps.wait_event(st.ring_free[slot])
    J = int(st.amplitudes_host.shape[0])
    size = int(np.prod(st.amplitudes_host.shape[1:]))
    _native.check(lib.ptycho_gather_patterns(
        ctypes.c_void_p(st.amp_mapped), J, size,
        ctypes.c_void_p(st.order.data_ptr() + 4 * start), end - start,
        ctypes.c_void_p(st.amp_ring[slot].data_ptr()), ctypes.c_void_p(ps.cuda_stream)))
    st.ring_ready[slot].record(ps)
    st.launches += 1


def run_batch(st: DeviceState, start: int, end: int, host_order: np.ndarray, *,
              projection=False, step_size=0.5, normalization_min=1.0, fix_probe=False,
              projection_abc=(0.0, 0.0, 0.0), position_correction=None, amplitudes=None):
    """amplitudes: (pointer, rows pointer) of the batch's patterns when the caller
    staged them; else taken from the state."""
    lib = _native.lib()
    n = end - start
    rows_ptr = ctypes.c_void_p(st.order.data_ptr() + 4 * start)
    if amplitudes is not None:
        amps_ptr, amp_rows = amplitudes
    else:
        amps_ptr, amp_rows = _batch_amplitudes(st, start, end, host_order)
    g = ctypes.byref(st.geometry)
    props = _ptr(st.propagators)
    if projection:
        a, b, c = projection_abc
        status = lib.ptycho_projection_batch(
            g, _ptr(st.object), _ptr(st.probe), amps_ptr, amp_rows, _ptr(st.positions),
            rows_ptr, n, float(a), float(b), float(c), float(normalization_min),
            1 if fix_probe else 0, _ptr(st.exit_waves), 1 if st.exit_waves_valid else 0,
            props, _ptr(st.error_accum), _ws_ptr(st), st.workspace_bytes, _stream())
    else:
        status = lib.ptycho_gd_batch(
            g, _ptr(st.object), _ptr(st.probe), amps_ptr, amp_rows, _ptr(st.positions),
            rows_ptr, n, float(step_size), float(normalization_min), 1 if fix_probe else 0,
            _ptr(st.det_mask), props, _ptr(st.error_accum), _ws_ptr(st), st.workspace_bytes,
            _stream())
    _native.check(status)
    st.launches += 5 if fix_probe else 8
    if position_correction is not None:
        pc = position_correction
        none = -1.0
        status = lib.ptycho_position_correction(
            g, _ptr(st.object), _ptr(st.probe), props, amps_ptr, amp_rows, _ptr(st.positions),
            _ptr(st.positions_initial), rows_ptr, n, float(pc["step_size"]),
            none if pc["max_update_px"] is None else float(pc["max_update_px"]),
            none if pc["max_total_px"] is None else float(pc["max_total_px"]),
            _ws_ptr(st), st.workspace_bytes, _stream())
        _native.check(status)
        st.launches += 1


def positions_com_constraint(st: DeviceState) -> None:
    """positions -= mean(positions) - mean(initial positions)
    (ptychographic_constraints.py:1292-1311)."""
    st.positions -= st.positions.mean(0) - st.positions_initial.mean(0)


def positions_affine_constraint(st: DeviceState, initial_positions: np.ndarray):
    """positions <- the RANSAC affine map of the initial positions that best fits
    them (ptychographic_constraints.py:1313-1350), fitted on the host from the
    device positions (NumPy's global generator draws the subsets, between the
    batch shuffles as in the reference); returns the transform."""
    from .positions import affine_constraint

    torch = _torch()
    new, tf = affine_constraint(initial_positions, st.positions.cpu().numpy())
    st.positions.copy_(torch.from_numpy(np.ascontiguousarray(new, dtype=np.float32)))
    return tf


def self_consistency_errors(st: DeviceState, max_batch: int) -> np.ndarray:
    """Per-position sum (A - |F|)^2 of a forward-only pass over the positions in
    natural order, batch by batch (ptychographic_methods.py:2227-2291); float32."""
    torch = _torch()
    lib = _native.lib()
    J = int(st.positions.shape[0])
    natural = np.arange(J)
    st.order.copy_(torch.arange(J, dtype=torch.int32, device=st.order.device))
    out = torch.empty(J, dtype=torch.float32, device=st.order.device)
    g = ctypes.byref(st.geometry)
    for start, end in generate_batches(J, max_batch):
        amps_ptr, amp_rows = _batch_amplitudes(st, start, end, natural)
        rows_ptr = ctypes.c_void_p(st.order.data_ptr() + 4 * start)
        _native.check(lib.ptycho_self_consistency_errors(
            g, _ptr(st.object), _ptr(st.probe), amps_ptr, amp_rows, _ptr(st.positions),
            rows_ptr, end - start, _ptr(st.propagators),
            ctypes.c_void_p(out.data_ptr() + 4 * start), _ws_ptr(st), st.workspace_bytes,
            _stream()))
        st.launches += 2
    return out.cpu().numpy()


def upload_order(st: DeviceState, host_order: np.ndarray) -> None:
    """Copy the iteration's position order to the device through one of two pinned
    buffers and an asynchronous copy on the current stream: the call returns at
    once and the caller may reuse (shuffle) its array while the GPU still works."""
    torch = _torch()
    n = int(host_order.shape[0])
    if st.order_pinned is None:
        cap = int(st.order.shape[0])
        st.order_pinned = [torch.empty(cap, dtype=torch.int32, pin_memory=True)
                           for _ in range(2)]
        st.order_events = [None, None]
    k = st.order_turn
    st.order_turn ^= 1
    if st.order_events[k] is not None:
        st.order_events[k].synchronize()  # the copy out of this buffer has run
    st.order_pinned[k].numpy()[:n] = host_order
    st.order[:n].copy_(st.order_pinned[k][:n], non_blocking=True)
    ev = torch.cuda.Event()
    ev.record()
    st.order_events[k] = ev


def stage_first_batch(st: DeviceState, max_batch: int) -> None:
    """Gather the first batch's patterns of the order in st.order into ring slot 0
    on the prefetch stream, after everything issued so far on the current stream
    (page-locked host amplitudes only). The transfer then runs while the host
    prepares the iteration; the current stream waits for it (ring_ready[0])
    before the iteration, which runs with first_staged=True."""
    torch = _torch()
    n = int(st.positions.shape[0])
    start, end = next(iter(generate_batches(n, max_batch)))
    st.prefetch_stream.wait_stream(torch.cuda.current_stream())
    st.ring_free[0].record(st.prefetch_stream)
    _gather_batch(st, 0, start, end)


def run_iteration(st: DeviceState, host_order: Optional[np.ndarray], max_batch: int,
                  first_staged: bool = False, **kw) -> None:
    """One pass over all positions in `host_order` (already shuffled), batch by batch.
    The batch errors accumulate into st.error_accum (float32 on the device).
    host_order=None uses the order already in st.order (no host transfer: the
    form that a CUDA graph can capture; device-resident or page-locked amplitudes).
    first_staged: the first batch's patterns are already in ring slot 0
    (stage_first_batch) and the current stream has waited for them."""
    torch = _torch()
    if host_order is None:
        if st.amplitudes is None and st.amp_mapped is None:
            raise ValueError("an iteration without a host order needs device-resident or "
                             "page-locked amplitudes")
        n = int(st.positions.shape[0])
    else:
        n = int(host_order.shape[0])
        upload_order(st, host_order)
    st.error_accum.zero_()
    # batch chaining: each batch computes the next batch's probe spectrum right
    # after its probe update (concurrently with the object update); with a fixed
    # probe the first batch's spectrum serves them all. Position correction reads
    # the batch's own spectrum after the update, so it does not chain.
    batches = list(generate_batches(n, max_batch))
    fixed = bool(kw.get("fix_probe"))
    chain = not fixed and kw.get("position_correction") is None
    base = st.geometry.flags & ~(_native.FLAG_SPECTRUM_READY | _native.FLAG_PREPARE_SPECTRUM)
    ring = st.amp_ring is not None
    if ring:
        # both slots are free once everything issued so far on this stream is done
        # (this also orders the gathers after the order upload)
        cur = torch.cuda.current_stream()
        for ev in st.ring_free:
            ev.record(cur)
        if not first_staged:
            _gather_batch(st, 0, *batches[0])
    try:
        for i, (start, end) in enumerate(batches):
            flags = base
            if i > 0 and (chain or fixed):
                flags |= _native.FLAG_SPECTRUM_READY
            if chain and i + 1 < len(batches):
                flags |= _native.FLAG_PREPARE_SPECTRUM
            st.geometry.flags = flags
            amps = None
            if ring:
                slot = i & 1
                if i + 1 < len(batches):
                    _gather_batch(st, slot ^ 1, *batches[i + 1])
                if i > 0 or not first_staged:
                    cur.wait_event(st.ring_ready[slot])
                amps = (ctypes.c_void_p(st.amp_ring[slot].data_ptr()), None)
            run_batch(st, start, end, host_order, amplitudes=amps, **kw)
            if ring:
                st.ring_free[slot].record(cur)
    finally:
        st.geometry.flags = base
    if kw.get("projection"):
        st.exit_waves_valid = True


def object_constraints(st: DeviceState, *, shrinkage_rad: float, use_mask: bool,
                       pure_phase: bool, positivity: bool) -> None:
    lib = _native.lib()
    apply_shrinkage = shrinkage_rad > 0.0 or use_mask
    mask = _ptr(st.fov_mask_inverse) if use_mask else None
    _native.check(lib.ptycho_object_constraints(
        ctypes.byref(st.geometry), _ptr(st.object), mask, float(shrinkage_rad),
        1 if apply_shrinkage else 0, 1 if pure_phase else 0, 1 if positivity else 0,
        _ws_ptr(st), st.workspace_bytes, _stream()))
    st.launches += 3 if use_mask else 1


def probe_com_constraint(st: DeviceState) -> None:
    lib = _native.lib()
    _native.check(lib.ptycho_probe_com_constraint(
        ctypes.byref(st.geometry), _ptr(st.probe), _ws_ptr(st), st.workspace_bytes, _stream()))
    st.launches += 3


def probe_orthogonalization(st: DeviceState, on_device: bool = False) -> None:
    """Gram matrix on the GPU, eigh of the M x M matrix on the host, mixing on the GPU
    (ptychographic_constraints.py:1181-1216). Modes are ordered by decreasing
    intensity; the intensity of mode i is the i-th eigenvalue.

    on_device=True runs the eigen-decomposition on the GPU too (no host round
    trip, capturable in a CUDA graph); its eigenvectors carry a fixed phase
    convention, so modes may differ from the host path by one phase per mode."""
    torch = _torch()
    lib = _native.lib()
    g = ctypes.byref(st.geometry)
    if on_device:
        _native.check(lib.ptycho_probe_orthogonalize(g, _ptr(st.probe), _ws_ptr(st),
                                                      st.workspace_bytes, _stream()))
        st.launches += 3
        return
    _native.check(lib.ptycho_probe_gram(g, _ptr(st.probe), _ptr(st.gram), _stream()))
    gram = st.gram.cpu().numpy()
    upper = np.triu(gram)
    evals, evecs = np.linalg.eigh(upper.astype(np.complex64), UPLO="U")
    coeffs = evecs.T  # new mode i = sum_j evecs[j, i] P_j
    # |new mode i|^2 = e_i^H G e_i = eigenvalue i: sort by decreasing intensity
    order = np.argsort(evals, axis=None)[::-1]
    coeffs = np.ascontiguousarray(coeffs[order], dtype=np.complex64)
    st.coeffs.copy_(torch.from_numpy(coeffs))
    _native.check(lib.ptycho_probe_mix(g, _ptr(st.probe), _ptr(st.coeffs),
                                       _ptr(st.probe_tmp), _stream()))
    st.probe.copy_(st.probe_tmp)
    st.launches += 2


def read_error(st: DeviceState) -> np.float32:
    """The iteration's error sum (one device-to-host synchronisation). Raises
    _native.PtychoError (a RuntimeError) with status PTYCHO_ERR_NONFINITE when it
    is NaN or infinite: a non-finite scan position, amplitude, probe or object
    value, or an update that overflowed."""
    value = ctypes.c_float(0.0)
    _native.check(_native.lib().ptycho_read_error(_ptr(st.error_accum), ctypes.byref(value),
                                                  _stream()))
    return np.float32(value.value)


class IterationDriver:
    """Runs reconstruction iterations on a DeviceState: all batches of the
    shuffled order, then the per-iteration constraints; the error is read back
    (one device-to-host sync) only when asked for."""

    def __init__(self, st: DeviceState, *, max_batch, projection=False, step_size=0.5,
                 normalization_min=1.0, fix_probe=False, projection_abc=(0.0, 0.0, 0.0),
                 shrinkage_rad=0.0, use_mask=False, pure_phase=False, positivity=True,
                 fix_probe_com=True, orthogonalize_probe=False, mean_intensity=1.0,
                 position_correction=None, device_orthogonalization=False,
                 graph=False, identical_slices=False, probe_aperture=None,
                 probe_amplitude_mask=None, gaussian=None, object_constraints=True):
        """probe_aperture: (Sx, Sy) Fourier amplitude of the initial probe (mode 0)
        for the aperture constraint; probe_amplitude_mask: (Sx, Sy) real-space mask
        of the amplitude constraint; identical_slices: average the object slices;
        gaussian: (float64 weights of length 2 R + 1, pure_phase) of the object blur;
        object_constraints=False leaves the object constraints to the caller (the
        tomography volume)."""
        self.st = st
        torch = _torch()
        dev = st.object.device
        self.object_constraints = bool(object_constraints)

        def dev_f32(a):
            if a is None:
                return None
            return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)

        self.identical_slices = bool(identical_slices) and st.geometry.num_slices > 1
        self.probe_aperture = dev_f32(probe_aperture)
        self.probe_amplitude_mask = dev_f32(probe_amplitude_mask)
        self.gaussian = None
        if gaussian is not None:
            weights, pure = gaussian
            w = torch.from_numpy(np.ascontiguousarray(weights, dtype=np.float64)).to(dev)
            scratch = torch.empty(4 * st.object.numel(), dtype=torch.float32, device=dev)
            self.gaussian = (w, (int(w.numel()) - 1) // 2, bool(pure), scratch)
        self.device_orthogonalization = bool(device_orthogonalization)
        self.graph = None
        self.calls = 0
        self._prefetched = None  # the order whose first batch prefetch() staged
        self.max_batch = int(max_batch)
        if position_correction is not None and st.positions_initial is None:
            raise ValueError("position correction needs a state created with positions_initial")
        self.batch_kw = dict(projection=projection, step_size=step_size,
                             normalization_min=normalization_min, fix_probe=fix_probe,
                             projection_abc=projection_abc,
                             position_correction=position_correction)
        self.positions_com = bool(position_correction and position_correction["center_of_mass"])
        self.positions_affine = bool(position_correction and position_correction.get("affine"))
        self.positions_initial_host = (st.positions_initial.cpu().numpy()
                                       if self.positions_affine else None)
        self.affine = None  # the last fitted AffineTransform
        self.shrinkage_rad = shrinkage_rad
        self.use_mask = use_mask
        self.pure_phase = pure_phase
        self.positivity = positivity
        self.fix_probe_com = fix_probe_com and not fix_probe
        self.orthogonalize = orthogonalize_probe and st.geometry.num_probes > 1
        self.mixed_state = bool(st.geometry.flags & _native.FLAG_MIXED_STATE)
        J = int(st.positions.shape[0])
        self.norm = np.float32(mean_intensity) * J
        # CUDA-graph replay of whole iterations: every kernel of an iteration in
        # one launch. Needs device-resident or page-locked amplitudes and, for
        # mixed states, the device eigen-decomposition (no host step inside).
        # host steps inside an iteration (the eigh of the mode orthogonalisation,
        # the affine fit of the positions) keep it out of a captured graph
        self.use_graph = bool(graph) and (st.amplitudes is not None or st.amp_mapped is not None) \
            and (not self.orthogonalize or self.device_orthogonalization) \
            and not self.positions_affine

    def _issue(self, first_staged: bool = False) -> None:
        st = self.st
        run_iteration(st, None, self.max_batch, first_staged=first_staged, **self.batch_kw)
        self._constraints()

    def prefetch(self, order: np.ndarray) -> None:
        """Start the next iteration's transfers for `order`: the order upload and,
        with page-locked host amplitudes, the first batch's pattern gather, so
        that they overlap the host work before iterate(order)."""
        st = self.st
        if st.amp_ring is None or order is None:
            return
        upload_order(st, order)
        stage_first_batch(st, self.max_batch)
        self._prefetched = np.array(order, copy=True)

    def iterate(self, order: Optional[np.ndarray]) -> None:
        """One iteration; order=None takes the order already in st.order."""
        st = self.st
        self.calls += 1
        ring = st.amp_ring is not None
        staged = self._prefetched is not None and order is not None and \
            np.array_equal(self._prefetched, order)
        self._prefetched = None
        if ring and order is not None and not staged:
            # page-locked host amplitudes: the first batch is gathered ahead of
            # the iteration, the others inside it one batch ahead
            upload_order(st, order)
            stage_first_batch(st, self.max_batch)
            staged = True
        if staged:
            _torch().cuda.current_stream().wait_event(st.ring_ready[0])
        if self.use_graph and order is not None:
            torch = _torch()
            if not ring:
                upload_order(st, order)
            if self.graph is None and self.calls >= 2:
                # the first iteration ran eagerly (library set-up for the stream);
                # capture the second on a side stream, then replay it from now on
                side = torch.cuda.Stream()
                _native.check(_native.lib().ptycho_prepare_stream(
                    ctypes.c_void_p(side.cuda_stream)))
                side.wait_stream(torch.cuda.current_stream())
                g = torch.cuda.CUDAGraph()
                before = st.launches
                with torch.cuda.graph(g, stream=side):
                    self._issue(first_staged=ring)
                torch.cuda.current_stream().wait_stream(side)
                self.graph = g
                self.graph_launches = st.launches - before
                st.launches -= self.graph_launches  # counted again at each replay
            if self.graph is not None:
                self.graph.replay()
                st.launches += self.graph_launches
            else:
                self._issue(first_staged=ring)
            if self.batch_kw.get("projection"):
                st.exit_waves_valid = True
            return
        if staged:
            run_iteration(st, None, self.max_batch, first_staged=True, **self.batch_kw)
        else:
            run_iteration(st, order, self.max_batch, **self.batch_kw)
        self._constraints()

    def _constraints(self) -> None:
        # order of ptychographic_constraints.py:649-726 (objects) and 1091-1148,
        # 1218-1285 (probes)
        st = self.st
        lib = _native.lib()
        if self.gaussian is not None:
            w, radius, pure, scratch = self.gaussian
            _native.check(lib.ptycho_object_gaussian_constraint(
                ctypes.byref(st.geometry), _ptr(st.object), _ptr(w), radius, 1 if pure else 0,
                _ptr(scratch), _stream()))
            st.launches += 2 + (3 if st.geometry.num_slices > 1 else 2)
        if self.identical_slices:
            _native.check(lib.ptycho_object_identical_slices(
                ctypes.byref(st.geometry), _ptr(st.object), _stream()))
            st.launches += 1
        if self.object_constraints:
            object_constraints(st, shrinkage_rad=self.shrinkage_rad, use_mask=self.use_mask,
                               pure_phase=self.pure_phase, positivity=self.positivity)
        if self.fix_probe_com:
            probe_com_constraint(st)
        if self.probe_aperture is not None:
            _native.check(lib.ptycho_probe_aperture_constraint(
                ctypes.byref(st.geometry), _ptr(st.probe), _ptr(self.probe_aperture),
                _stream()))
            st.launches += 1
        if self.probe_amplitude_mask is not None:
            _native.check(lib.ptycho_probe_amplitude_constraint(
                ctypes.byref(st.geometry), _ptr(st.probe), _ptr(self.probe_amplitude_mask),
                _stream()))
            st.launches += 1
        if self.orthogonalize:
            probe_orthogonalization(st, on_device=self.device_orthogonalization)
        if self.positions_com:
            positions_com_constraint(st)
        if self.positions_affine:
            self.affine = positions_affine_constraint(st, self.positions_initial_host)

    def error(self) -> np.float32:
        """Normalised error of the last iteration: float32 sum over batches divided
        by mean intensity x J (singleslice_ptychography.py:929-932)."""
        return np.float32(read_error(self.st) / self.norm)
