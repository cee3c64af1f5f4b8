"""ctypes binding of libtk_fdk.so (C ABI declared in include/tk_fdk.h).

The library is built in-tree by ``tomokvas_gb300._build.build()`` (or
``__graft_entry__.build()``).  There is no fallback: if the shared library is
missing or cannot be loaded, every call raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes
import os

from ._build import LIB

TK_OK, TK_ERR_INVALID, TK_ERR_CUDA, TK_ERR_OOM, TK_ERR_STATE, TK_ERR_IO, TK_ERR_DEVICE, TK_ERR_UNSUPPORTED = range(8)
TK_WINDOW_RAMLAK, TK_WINDOW_SHEPP_LOGAN, TK_WINDOW_HANN = 0, 1, 2
TK_F32, TK_F16, TK_BF16, TK_F32_COEF = 0, 1, 2, 3
TK_LAYOUT_SINOGRAM, TK_LAYOUT_PROJECTION = 0, 1
TK_INPUT_F32, TK_INPUT_U16 = 0, 1
TK_FILTER_AUTO, TK_FILTER_FFT, TK_FILTER_TOEPLITZ = 0, 1, 2

WINDOWS = {"ramlak": TK_WINDOW_RAMLAK, "shepp_logan": TK_WINDOW_SHEPP_LOGAN, "hann": TK_WINDOW_HANN}
PRECISIONS = {"f32": TK_F32, "f16": TK_F16, "bf16": TK_BF16, "f32c": TK_F32_COEF}
LAYOUTS = {"sinogram": TK_LAYOUT_SINOGRAM, "projection": TK_LAYOUT_PROJECTION}

# Every symbol include/tk_fdk.h declares (checked by the CPU test-suite).
EXPORTS = [
    "tk_version", "tk_last_error", "tk_get_free_mem_info", "tk_pad_length", "tk_default_zoff",
    "tk_zblock_offsets", "tk_device_error_flags", "tk_filter_projections", "tk_backproject",
    "tk_filtered_bytes", "tk_fdk_workspace_bytes", "tk_fdk_device", "tk_fdk_device_noalloc",
    "tk_fdk_stream_workspace_bytes", "tk_fdk_stream",
    "tk_forward_project", "tk_filter_transpose", "tk_fdk_forward", "tk_fdk_backward", "tk_phantom_project", "tk_bp_variant_count",
    "tk_bp_variant_name", "tk_bp_variant_precision", "tk_bp_select_variant", "tk_fp_select_variant", "tk_fdk_create", "tk_fdk_destroy",
    "tk_fdk_set_gpu_id", "tk_fdk_set_block_size", "tk_fdk_set_allocation_limit", "tk_fdk_set_collecting",
    "tk_fdk_set_show_info", "tk_fdk_show_info", "tk_fdk_set_axis_direction", "tk_fdk_set_sinogram_properties",
    "tk_fdk_set_reconstruction_properties", "tk_fdk_set_scale_xyz", "tk_fdk_set_projections_u16",
    "tk_fdk_set_input_layout", "tk_fdk_set_filter", "tk_fdk_set_precision", "tk_fdk_set_stream",
    "tk_fdk_set_pipeline",
    "tk_fdk_initialize", "tk_fdk_calculate_reconstruction", "tk_fdk_reconstruct_device", "tk_fdk_get_timings",
    "tk_batch_create", "tk_batch_destroy", "tk_batch_set_precision", "tk_batch_submit", "tk_batch_size",
    "tk_batch_workspace_bytes", "tk_batch_plan", "tk_batch_run", "tk_batch_autotune", "tk_batch_variant_count",
    "tk_batch_variant_name", "tk_batch_variant", "tk_batch_select_variant",
    "tk_half_to_full_fan", "tk_half_to_parallel", "tk_kernel_launches", "tk_measure_fp32_fma_rate",
    "tk_filter_select_form", "tk_filter_form_for", "tk_batch_item_filter_form", "tk_batch_item_quarter_turn",
    "tk_batch_timings",
    "tk_refine_checkpoint_bytes", "tk_refine_workspace_bytes", "tk_refine_checkpoint", "tk_refine_volume",
    "tk_refine_step_size", "tk_diag_wait_timeout", "tk_diag_shrink_box",
]


class Geometry(ctypes.Structure):
    """Mirror of ``tk_geometry`` (include/tk_fdk.h)."""

    _fields_ = [
        ("W", ctypes.c_int), ("N", ctypes.c_int), ("H", ctypes.c_int),
        ("cX", ctypes.c_float), ("cZ", ctypes.c_float), ("dfi", ctypes.c_float),
        ("D", ctypes.c_float), ("tau", ctypes.c_float),
        ("X", ctypes.c_int), ("Y", ctypes.c_int), ("Z", ctypes.c_int),
        ("cx", ctypes.c_float), ("cy", ctypes.c_float), ("cz", ctypes.c_float),
        ("rot", ctypes.c_float), ("scale", ctypes.c_float),
        ("dirx", ctypes.c_int), ("diry", ctypes.c_int), ("dirz", ctypes.c_int),
    ]


class FlatField(ctypes.Structure):
    """Mirror of ``tk_flatfield``."""

    _fields_ = [
        ("dark", ctypes.c_void_p), ("flat", ctypes.c_void_p),
        ("dark_value", ctypes.c_float), ("flat_value", ctypes.c_float),
        ("A", ctypes.c_float), ("B", ctypes.c_float),
        ("invert", ctypes.c_int), ("floor_counts", ctypes.c_float),
    ]


BLOCK_SINK = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int)

_LIB = None


class TKError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"tk status {code}: {msg}")
        self.code = code


def load(path: str | None = None):
    """Load libtk_fdk.so; raise if it is not built (no CPU fallback exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = path or LIB
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(p)
    _declare(L)
    _LIB = L
    return L


def _declare(L):
    vp, ip, fp = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    G = ctypes.POINTER(Geometry)
    L.tk_version.restype = ip
    L.tk_last_error.restype = ctypes.c_char_p
    L.tk_get_free_mem_info.argtypes = [ip]
    L.tk_get_free_mem_info.restype = ctypes.c_size_t
    L.tk_pad_length.argtypes = [ip]
    L.tk_default_zoff.argtypes = [G]
    L.tk_default_zoff.restype = fp
    L.tk_zblock_offsets.argtypes = [G, ip, ctypes.POINTER(fp), ip]
    L.tk_device_error_flags.argtypes = [ctypes.POINTER(ctypes.c_uint), ip]
    L.tk_filter_projections.argtypes = [G, vp, ip, ip, ctypes.POINTER(FlatField), ip, vp, ip, vp, vp]
    L.tk_backproject.argtypes = [G, vp, ip, vp, ip, fp, vp, ip, vp]
    L.tk_filtered_bytes.argtypes = [G, ip]
    L.tk_filtered_bytes.restype = ctypes.c_size_t
    L.tk_fdk_workspace_bytes.argtypes = [G, ip]
    L.tk_fdk_workspace_bytes.restype = ctypes.c_size_t
    L.tk_fdk_device.argtypes = [G, vp, ip, ip, ctypes.POINTER(FlatField), ip, ip, vp, ctypes.c_size_t, vp, vp]
    L.tk_forward_project.argtypes = [G, vp, ip, fp, vp, ip, vp]
    L.tk_filter_transpose.argtypes = [G, vp, ip, vp, ip, vp]
    L.tk_fdk_forward.argtypes = [G, vp, ip, ip, vp, ctypes.c_size_t, vp, vp]
    L.tk_fdk_backward.argtypes = [G, vp, ip, ip, vp, ctypes.c_size_t, vp, vp]
    L.tk_fdk_stream_workspace_bytes.argtypes = [G, ip, ip, ip]
    L.tk_fdk_stream_workspace_bytes.restype = ctypes.c_size_t
    L.tk_fdk_stream.argtypes = [G, vp, ip, ctypes.POINTER(FlatField), ip, ip, ip, vp, ctypes.c_size_t, vp, vp]
    L.tk_fdk_device_noalloc.argtypes = [G, vp, ip, ip, ctypes.POINTER(FlatField), ip, ip, vp, vp]
    L.tk_phantom_project.argtypes = [G, ctypes.POINTER(ctypes.c_double), ip, ip, vp, vp]
    L.tk_bp_variant_count.restype = ip
    L.tk_bp_variant_name.argtypes = [ip]
    L.tk_bp_variant_name.restype = ctypes.c_char_p
    L.tk_bp_variant_precision.argtypes = [ip]
    L.tk_bp_select_variant.argtypes = [ip]
    L.tk_fp_select_variant.argtypes = [ip]
    L.tk_filter_select_form.argtypes = [ip]
    L.tk_filter_form_for.argtypes = [ip, ip]
    L.tk_batch_item_filter_form.argtypes = [vp, ip]
    L.tk_batch_item_quarter_turn.argtypes = [vp, ip]
    L.tk_batch_timings.argtypes = [vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    L.tk_refine_checkpoint_bytes.argtypes = [G, ip]
    L.tk_refine_checkpoint_bytes.restype = ctypes.c_size_t
    L.tk_refine_workspace_bytes.argtypes = [G]
    L.tk_refine_workspace_bytes.restype = ctypes.c_size_t
    L.tk_refine_checkpoint.argtypes = [G, vp, ip, ip, ctypes.POINTER(FlatField), ip, vp, ip, vp, ctypes.c_size_t, vp]
    L.tk_refine_volume.argtypes = [G, vp, ip, fp, ip, vp, vp, vp, ctypes.c_size_t, vp]
    L.tk_refine_step_size.argtypes = [G, ip, vp, vp, ctypes.c_size_t, ctypes.POINTER(fp), vp]
    L.tk_diag_wait_timeout.argtypes = [ctypes.c_double, vp]
    L.tk_diag_shrink_box.argtypes = [ip]
    L.tk_batch_create.argtypes = [ctypes.POINTER(vp)]
    L.tk_batch_destroy.argtypes = [vp]
    L.tk_batch_destroy.restype = None
    L.tk_batch_set_precision.argtypes = [vp, ip]
    L.tk_batch_submit.argtypes = [vp, G, vp, ip, ip, ctypes.POINTER(FlatField), ip, vp]
    L.tk_batch_size.argtypes = [vp]
    L.tk_batch_workspace_bytes.argtypes = [vp]
    L.tk_batch_workspace_bytes.restype = ctypes.c_size_t
    L.tk_batch_plan.argtypes = [vp, vp, ctypes.c_size_t, vp]
    L.tk_batch_run.argtypes = [vp, ip, vp]
    L.tk_batch_autotune.argtypes = [vp, vp, ctypes.POINTER(ip), ctypes.POINTER(fp)]
    L.tk_batch_variant_name.argtypes = [ip]
    L.tk_batch_variant_name.restype = ctypes.c_char_p
    L.tk_batch_variant.argtypes = [vp]
    L.tk_batch_select_variant.argtypes = [vp, ip]
    L.tk_kernel_launches.restype = ctypes.c_ulonglong
    L.tk_measure_fp32_fma_rate.argtypes = [ctypes.POINTER(ctypes.c_double)]
    dd = ctypes.c_double
    L.tk_half_to_full_fan.argtypes = [vp, ip, ip, ip, ip, dd, dd, ip, vp, vp]
    L.tk_half_to_parallel.argtypes = [vp, ip, ip, ip, ip, dd, dd, vp, vp]
    H = vp
    L.tk_fdk_create.argtypes = [ctypes.POINTER(vp)]
    L.tk_fdk_destroy.argtypes = [H]
    L.tk_fdk_destroy.restype = None
    for name, args in [
        ("tk_fdk_set_gpu_id", [ip]), ("tk_fdk_set_block_size", [ip]),
        ("tk_fdk_set_allocation_limit", [ctypes.c_longlong]), ("tk_fdk_set_collecting", [ip]),
        ("tk_fdk_set_show_info", [ip]), ("tk_fdk_show_info", []), ("tk_fdk_set_axis_direction", [ip, ip, ip]),
        ("tk_fdk_set_sinogram_properties", [vp, ip, fp, ip, ip, fp, fp, fp, fp]),
        ("tk_fdk_set_reconstruction_properties", [ip, fp, ip, fp, ip, fp, fp]),
        ("tk_fdk_set_scale_xyz", [fp]),
        ("tk_fdk_set_projections_u16", [vp, ip, vp, vp, fp, fp, fp, fp, ip, fp]),
        ("tk_fdk_set_input_layout", [ip]), ("tk_fdk_set_filter", [ip]), ("tk_fdk_set_precision", [ip]),
        ("tk_fdk_set_stream", [vp]), ("tk_fdk_set_pipeline", [ip]), ("tk_fdk_initialize", []),
        ("tk_fdk_calculate_reconstruction", [BLOCK_SINK, vp]), ("tk_fdk_reconstruct_device", [vp]),
        ("tk_fdk_get_timings", [ctypes.POINTER(fp)] * 4),
    ]:
        getattr(L, name).argtypes = [H] + args
        getattr(L, name).restype = ip


def check(rc: int):
    if rc != TK_OK:
        raise TKError(rc, load().tk_last_error().decode(errors="replace"))
    return rc
