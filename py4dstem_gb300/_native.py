"""ctypes binding of libptycho_gb300.so (the C ABI in include/ptycho_gb300.h).

The library is the only compute path of this package: there is no CPU fallback.
If it cannot be loaded, :func:`lib` raises ``RuntimeError``.
"""

from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

PTYCHO_OK = 0
PTYCHO_ERR_NONFINITE = 5
FLAG_MIXED_STATE = 1
FLAG_KEEP_FARFIELD = 2
FLAG_SPECTRUM_READY = 4
FLAG_PREPARE_SPECTRUM = 8
_STATUS_NAMES = {
    1: "invalid argument",
    2: "unsupported geometry",
    3: "workspace",
    4: "CUDA error",
    5: "non-finite value",
}


class PtychoError(RuntimeError):
    """A libptycho_gb300 call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"libptycho_gb300: {_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Geometry(ctypes.Structure):
    _fields_ = [
        ("roi_x", ctypes.c_int32),
        ("roi_y", ctypes.c_int32),
        ("object_x", ctypes.c_int32),
        ("object_y", ctypes.c_int32),
        ("num_slices", ctypes.c_int32),
        ("num_probes", ctypes.c_int32),
        ("object_is_potential", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("detector_x", ctypes.c_int32),   # 0: the ROI shape (no resampling)
        ("detector_y", ctypes.c_int32),
    ]


_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_f32 = ctypes.c_float
_sz = ctypes.c_size_t
_f64 = ctypes.c_double

_SIGNATURES = {
    "ptycho_abi_version": ([], ctypes.c_int),
    "ptycho_last_error": ([], ctypes.c_char_p),
    "ptycho_roi_supported": ([_i32, _i32], ctypes.c_int),
    "ptycho_geometry_supported": ([ctypes.POINTER(Geometry)], ctypes.c_int),
    "ptycho_workspace_bytes": ([ctypes.POINTER(Geometry), _i32], _sz),
    "ptycho_gd_batch": (
        [ctypes.POINTER(Geometry), _vp, _vp, _vp, _vp, _vp, _vp, _i32, _f32, _f32, _i32,
         _vp, _vp, _vp, _vp, _sz, _vp],
        ctypes.c_int,
    ),
    "ptycho_projection_batch": (
        [ctypes.POINTER(Geometry), _vp, _vp, _vp, _vp, _vp, _vp, _i32, _f32, _f32, _f32,
         _f32, _i32, _vp, _i32, _vp, _vp, _vp, _sz, _vp],
        ctypes.c_int,
    ),
    "ptycho_object_constraints": (
        [ctypes.POINTER(Geometry), _vp, _vp, _f32, _i32, _i32, _i32, _vp, _sz, _vp],
        ctypes.c_int,
    ),
    "ptycho_probe_com_constraint": (
        [ctypes.POINTER(Geometry), _vp, _vp, _sz, _vp], ctypes.c_int),
    "ptycho_probe_gram": ([ctypes.POINTER(Geometry), _vp, _vp, _vp], ctypes.c_int),
    "ptycho_probe_mix": ([ctypes.POINTER(Geometry), _vp, _vp, _vp, _vp], ctypes.c_int),
    "ptycho_probe_orthogonalize": ([ctypes.POINTER(Geometry), _vp, _vp, _sz, _vp], ctypes.c_int),
    "ptycho_prepare_stream": ([_vp], ctypes.c_int),
    "ptycho_mapped_host_pointer": ([_vp, _sz, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "ptycho_gather_patterns": ([_vp, _i32, ctypes.c_int64, _vp, _i32, _vp, _vp], ctypes.c_int),
    "ptycho_enable_kernel_timing": ([_i32], ctypes.c_int),
    "ptycho_kernel_timing": ([ctypes.POINTER(_f32), ctypes.POINTER(_i32)], ctypes.c_int),
    "ptycho_fp32_fma_probe": ([_i32, _i32, _vp, _vp], ctypes.c_int),
    "ptycho_set_kernel_schedule": ([_i32, _i32], ctypes.c_int),
    "ptycho_position_correction": (
        [ctypes.POINTER(Geometry), _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _f32, _f64,
         _f64, _vp, _sz, _vp],
        ctypes.c_int,
    ),
    "ptycho_gd_gradient": (
        [ctypes.POINTER(Geometry), _vp, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _vp, _vp,
         _vp, _sz, _vp],
        ctypes.c_int,
    ),
    "ptycho_self_consistency_errors": (
        [ctypes.POINTER(Geometry), _vp, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _sz, _vp],
        ctypes.c_int,
    ),
    "ptycho_object_identical_slices": ([ctypes.POINTER(Geometry), _vp, _vp], ctypes.c_int),
    "ptycho_object_gaussian_constraint": (
        [ctypes.POINTER(Geometry), _vp, _vp, _i32, _i32, _vp, _vp], ctypes.c_int),
    "ptycho_probe_aperture_constraint": (
        [ctypes.POINTER(Geometry), _vp, _vp, _vp], ctypes.c_int),
    "ptycho_probe_amplitude_constraint": (
        [ctypes.POINTER(Geometry), _vp, _vp, _vp], ctypes.c_int),
    "ptycho_pattern_com": ([_vp, _i32, _i32, _i32, _vp, _i32, _vp, _vp, _vp], ctypes.c_int),
    "ptycho_rotation_search": (
        [_vp, _vp, _i32, _i32, _i32, _vp, _vp, _i32, _i32, _vp, _vp], ctypes.c_int),
    "ptycho_normalize_patterns": (
        [_vp, _i32, _i32, _vp, _i32, _vp, _vp, _i32, _vp, _vp, _vp], ctypes.c_int),
    "ptycho_probe_overlap": (
        [ctypes.POINTER(Geometry), _vp, _vp, _i32, _i32, _vp, _vp, _sz, _vp], ctypes.c_int),
    "ptycho_volume_rotate": (
        [_vp, _i32, _vp, _i32, _i32, _i32, _i32, _vp, _vp, _vp, _sz, _vp], ctypes.c_int),
    "ptycho_volume_project": ([_vp, _i32, _i32, _i32, _i32, _vp, _vp], ctypes.c_int),
    "ptycho_volume_expand_update": (
        [_vp, _vp, _i32, _i32, _i32, _i32, _vp, _i32, _vp], ctypes.c_int),
    "ptycho_volume_add_scaled": ([_vp, _vp, ctypes.c_int64, _i32, _vp], ctypes.c_int),
    "ptycho_volume_constraints": ([_vp, ctypes.c_int64, _f32, _i32, _i32, _vp], ctypes.c_int),
    "ptycho_read_error": ([_vp, ctypes.POINTER(_f32), _vp], ctypes.c_int),
    "ptycho_nn_gemm_bf16": ([_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp], ctypes.c_int),
    "ptycho_nn_conv3x3_forward": (
        [_vp, _i32, _i32, _i32, _i32, _vp, _vp, _i32, _i32, _vp, _vp, _vp], ctypes.c_int),
    "ptycho_nn_conv3x3_backward_data": (
        [_vp, _i32, _i32, _i32, _i32, _vp, _i32, _vp, _vp, _vp], ctypes.c_int),
    "ptycho_nn_conv3x3_wgrad_workspace_bytes": ([_i32, _i32, _i32, _i32, _i32], _sz),
    "ptycho_nn_conv3x3_backward_weight": (
        [_vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp, _vp, _vp, _sz, _vp, _vp], ctypes.c_int),
    "ptycho_nn_unet_param_bytes": ([], _sz),
    "ptycho_nn_unet_param_offset": ([_i32, _i32], ctypes.c_int64),
    "ptycho_nn_unet_workspace_bytes": ([_i32, _i32, _i32], _sz),
    "ptycho_nn_unet_init": ([_vp, ctypes.c_uint64, _vp], ctypes.c_int),
    "ptycho_nn_unet_forward": ([_vp, _vp, _i32, _i32, _i32, _vp, _vp, _sz, _vp], ctypes.c_int),
    "ptycho_nn_unet_train_step": (
        [_vp, _vp, _vp, _vp, _f32, _i32, _i32, _i32, _f32, _i32, _vp, _vp, _sz, _vp],
        ctypes.c_int),
    "ptycho_nn_check": ([_vp, _i32, _i32, _i32, _vp], ctypes.c_int),
    "ptycho_nn_last_error": ([], ctypes.c_char_p),
    "ptycho_nn_lattice_objects": ([_i32, _i32, _f32, _vp, _f32, _f32, _f32, _vp, _vp, _vp,
                                   _vp], ctypes.c_int),
    "ptycho_nn_scan_images": (
        [_i32, _i32, _i32, _vp, _vp, _vp, _vp, _f32, _f32, ctypes.c_uint64, _vp, _vp, _vp, _vp,
         _vp], ctypes.c_int),
    "ptycho_nn_virtual_images": ([_vp, _i32, _i32, _i32, _f32, _vp, _vp, _vp, _vp],
                                 ctypes.c_int),
    "ptycho_gd_batch_noalloc": (
        [ctypes.POINTER(Geometry), _vp, _vp, _vp, _vp, _vp, _vp, _i32, _f32, _f32, _i32,
         _vp, _vp, _vp, _vp],
        ctypes.c_int,
    ),
}

EXPORTED_SYMBOLS = tuple(_SIGNATURES)

_LOCK = threading.Lock()
_LIB = None


def library_path() -> str:
    return _build.LIB_PATH


def load_library(path: str | None = None, build_if_missing: bool = True):
    """Load the shared library (building it in-tree first when it is stale and
    nvcc is available) and attach the C signatures."""
    path = path or library_path()
    if build_if_missing and path == library_path():
        try:
            _build.build()
        except RuntimeError:
            if not os.path.exists(path):
                raise
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing; build it with `python -m py4dstem_gb300.build` "
            "(this package has no CPU compute path)")
    handle = ctypes.CDLL(path)
    for name, (args, res) in _SIGNATURES.items():
        fn = getattr(handle, name)
        fn.argtypes = args
        fn.restype = res
    return handle


def lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            _LIB = load_library()
        return _LIB


def check(status: int) -> None:
    if status != PTYCHO_OK:
        msg = lib().ptycho_last_error().decode(errors="replace")
        raise PtychoError(status, msg)
