"""Device half of ``preprocess()`` when the reconstruction runs on the GPU.

The per-pattern work of the preprocessing runs in libptycho_gb300 on the
device copy of the diffraction intensities:

=====================================  ==============================  =====================================
step                                   entry point                     reference (py4DSTEM 0.14.18)
=====================================  ==============================  =====================================
centre of mass of every pattern        ``ptycho_pattern_com``          phase_base_class.py:613-700
rotation search (curl / divergence)    ``ptycho_rotation_search``      phase_base_class.py:1086-1182
bilinear corner-centring, sqrt, sums   ``ptycho_normalize_patterns``   phase_base_class.py:1347-1460
probe-overlap map for the FOV mask     ``ptycho_probe_overlap``        singleslice_ptychography.py:504-540
=====================================  ==============================  =====================================

The surface fit of the centre of mass (scipy ``curve_fit`` over one value per
scan position), the arg-min over angles, the running float32 sum of the pattern
sums and the Gaussian blur of the overlap map stay on the host, as the same
NumPy/SciPy calls the host path makes. The kernels reproduce NumPy's float32
summation order and single roundings, so the centre of mass, the rotation
values and the amplitudes carry the bits of the host path; the overlap map goes
through float32 FFTs and agrees to rounding.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .engine import _torch, make_geometry

_OVERLAP_BATCH = 1024


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(_torch().cuda.current_stream().cuda_stream)


def upload_intensities(intensities: np.ndarray):
    """(..., Qx, Qy) float32 host patterns -> contiguous (J, Qx, Qy) device tensor."""
    torch = _torch()
    arr = np.ascontiguousarray(intensities, dtype=np.float32)
    qx, qy = arr.shape[-2:]
    return torch.from_numpy(arr.reshape((-1, qx, qy))).to("cuda")


def pattern_com(intensities_dev, mask=None, vectorized=True):
    """(com_x, com_y) host arrays, one value per pattern, in the type NumPy gives
    pattern * mask: float32 without a mask or with a boolean / float32 / small
    integer mask; float64 for any other mask in the vectorised form; float32 with
    the float64 product rounded in place in the per-pattern form."""
    torch = _torch()
    J, qx, qy = intensities_dev.shape
    dev = intensities_dev.device
    mode, mask_dev = 0, None
    if mask is not None:
        m = np.asarray(mask)
        if np.result_type(np.float32, m.dtype) == np.float32:
            mode = 1
            mask_dev = torch.from_numpy(np.ascontiguousarray(m, dtype=np.float32)).to(dev)
        else:
            mode = 2 if vectorized else 3
            mask_dev = torch.from_numpy(np.ascontiguousarray(m, dtype=np.float64)).to(dev)
    out_t = torch.float64 if mode == 2 else torch.float32
    cx = torch.empty(J, dtype=out_t, device=dev)
    cy = torch.empty_like(cx)
    _native.check(_native.lib().ptycho_pattern_com(
        _ptr(intensities_dev), int(J), int(qx), int(qy),
        None if mask_dev is None else _ptr(mask_dev), mode, _ptr(cx), _ptr(cy), _stream()))
    return cx.cpu().numpy(), cy.cpu().numpy()


def rotation_values(com_x: np.ndarray, com_y: np.ndarray, cos_a: np.ndarray, sin_a: np.ndarray,
                    maximize_divergence: bool) -> np.ndarray:
    """(2, A): the mean |curl| (|div|) per angle, untransposed then transposed, in
    the type of the CoM field (float32, or float64 when the centre of mass was
    formed in float64)."""
    torch = _torch()
    r0, r1 = com_x.shape
    dbl = np.result_type(com_x.dtype, com_y.dtype, np.float32) == np.float64
    if r0 < 3 or r1 < 3:
        raise ValueError(
            f"the rotation search needs a scan of at least 3 x 3 positions (got {r0} x {r1}); "
            "pass force_com_rotation")
    dev = torch.device("cuda", torch.cuda.current_device())

    def up(a, dtype):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(dev)

    ft = np.float64 if dbl else np.float32
    nx, ny = up(com_x, ft), up(com_y, ft)
    c, s = up(np.ravel(cos_a), np.float32), up(np.ravel(sin_a), np.float32)
    A = int(c.numel())
    vals = torch.empty(2 * A, dtype=torch.float64 if dbl else torch.float32, device=dev)
    _native.check(_native.lib().ptycho_rotation_search(
        _ptr(nx), _ptr(ny), 1 if dbl else 0, int(r0), int(r1), _ptr(c), _ptr(s), A,
        1 if maximize_divergence else 0, _ptr(vals), _stream()))
    return vals.cpu().numpy().reshape(2, A)


def normalize_patterns(intensities_dev, com_fitted_x, com_fitted_y, positions_mask, crop_w):
    """Device amplitudes (J', Cx, Cy) and the float32 mean intensity.

    Patterns are taken in scan order, skipping those the positions mask leaves
    out; the mean is the float32 running sum of the shifted patterns' sums in
    that order divided by their number, as the host loop forms it."""
    torch = _torch()
    J, qx, qy = intensities_dev.shape
    dev = intensities_dev.device
    rows = None
    if positions_mask is not None:
        idx = np.flatnonzero(np.asarray(positions_mask, dtype=bool).ravel()).astype(np.int32)
        rows = torch.from_numpy(idx).to(dev)
        n_out = int(idx.size)
    else:
        n_out = int(J)
    cfx = torch.from_numpy(np.ascontiguousarray(com_fitted_x, dtype=np.float32).ravel()).to(dev)
    cfy = torch.from_numpy(np.ascontiguousarray(com_fitted_y, dtype=np.float32).ravel()).to(dev)
    if cfx.numel() != J:
        raise ValueError(f"{cfx.numel()} fitted centres for {J} patterns")
    cx_, cy_ = (2 * crop_w, 2 * crop_w) if crop_w else (qx, qy)
    amps = torch.empty((n_out, cx_, cy_), dtype=torch.float32, device=dev)
    sums = torch.empty(n_out, dtype=torch.float32, device=dev)
    _native.check(_native.lib().ptycho_normalize_patterns(
        _ptr(intensities_dev), int(qx), int(qy), None if rows is None else _ptr(rows), n_out,
        _ptr(cfx), _ptr(cfy), int(crop_w), _ptr(amps), _ptr(sums), _stream()))
    s = sums.cpu().numpy()
    # `mean += np.sum(shifted)` pattern by pattern in float32, then / count
    mean = np.add.accumulate(s, dtype=np.float32)[-1] if n_out else np.float32(0)
    mean = np.float32(mean) / n_out if n_out else np.float32(np.nan)
    return amps, mean


def probe_overlap(probe_single: np.ndarray, positions_px: np.ndarray, object_shape,
                  max_batch_size=None) -> np.ndarray:
    """(Px, Py) float32 probe-overlap map, summed on the device."""
    torch = _torch()
    lib = _native.lib()
    roi = probe_single.shape[-2:]
    if not lib.ptycho_roi_supported(int(roi[0]), int(roi[1])):
        raise NotImplementedError(
            f"no GPU kernel for a {roi[0]}x{roi[1]} region of interest "
            "(supported: square 32, 48, 64, 96, 128, 256 and 96 x 128, 128 x 96)")
    J = int(positions_px.shape[0])
    batch = max(1, min(int(max_batch_size or J), _OVERLAP_BATCH, J))
    geom = make_geometry(roi, object_shape, 1, 1, False)
    ws_bytes = int(lib.ptycho_workspace_bytes(ctypes.byref(geom), batch))
    if ws_bytes == 0:
        raise ValueError("invalid geometry for the probe-overlap workspace")
    dev = torch.device("cuda", torch.cuda.current_device())
    ws = torch.empty(ws_bytes + 256, dtype=torch.uint8, device=dev)
    base = ws.data_ptr()
    ws_ptr = ctypes.c_void_p((base + 255) // 256 * 256)
    probe = torch.from_numpy(np.ascontiguousarray(probe_single, dtype=np.complex64)).to(dev)
    pos = torch.from_numpy(np.ascontiguousarray(positions_px, dtype=np.float32)).to(dev)
    overlap = torch.empty(tuple(int(v) for v in object_shape), dtype=torch.float32, device=dev)
    _native.check(lib.ptycho_probe_overlap(
        ctypes.byref(geom), _ptr(probe), _ptr(pos), J, batch, _ptr(overlap), ws_ptr,
        ctypes.c_size_t(ws_bytes), _stream()))
    return overlap.cpu().numpy()
