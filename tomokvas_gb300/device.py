"""Stage API over device buffers (torch tensors used only as device memory).

Thin wrappers of the C ABI entry points tk_filter_projections,
tk_backproject, tk_fdk_device and tk_phantom_project.  All work runs in the
CUDA library; torch provides allocation and the current stream.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check, load


def _torch():
    import torch

    return torch


def _stream_ptr(stream=None) -> int:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _geom(g):
    return g.to_c() if hasattr(g, "to_c") else g


def row_pitch(W: int) -> int:
    return (W + 7) & ~7


def flatfield(flat=None, dark=None, flat_value=0.0, dark_value=0.0, A=1.0, B=0.0, invert=True, floor_counts=0.5):
    """tk_flatfield; flat/dark may be device tensors [H][W] (float32) or None."""
    ff = _lib.FlatField()
    ff.flat = None if flat is None else flat.data_ptr()
    ff.dark = None if dark is None else dark.data_ptr()
    ff.flat_value, ff.dark_value = float(flat_value), float(dark_value)
    ff.A, ff.B, ff.invert, ff.floor_counts = float(A), float(B), int(bool(invert)), float(floor_counts)
    ff._keep = (flat, dark)  # the device arrays must outlive every call that uses ff
    return ff


def filtered_bytes(g, precision=_lib.TK_F32) -> int:
    gc = _geom(g)
    return int(load().tk_filtered_bytes(ctypes.byref(gc), precision))


def alloc_filtered(g, precision=_lib.TK_F32, device="cuda"):
    """Device buffer for filtered projections in a storage format (see tk_precision)
    and its storage-scale word."""
    torch = _torch()
    if precision == _lib.TK_F32:
        q = torch.empty((g.N, g.H, row_pitch(g.W)), dtype=torch.float32, device=device)
    else:
        q = torch.empty(filtered_bytes(g, precision), dtype=torch.uint8, device=device)
    scale = torch.ones(1, dtype=torch.float32, device=device)
    return q, scale


def filter_projections(g, d_in, input_type=_lib.TK_INPUT_F32, layout=_lib.TK_LAYOUT_SINOGRAM, ff=None,
                       window=_lib.TK_WINDOW_RAMLAK, precision=_lib.TK_F32, out=None, stream=None):
    """Preprocess + ramp filter; returns (q [N][H][Wp], scale[1]) device tensors."""
    L = load()
    q, scale = out if out is not None else alloc_filtered(g, precision, d_in.device)
    gc = _geom(g)
    check(L.tk_filter_projections(ctypes.byref(gc), d_in.data_ptr(), input_type, layout,
                                  None if ff is None else ctypes.byref(ff), window, q.data_ptr(), precision,
                                  scale.data_ptr(), _stream_ptr(stream)))
    return q, scale


def backproject(g, q, scale, precision=_lib.TK_F32, vol=None, nz=None, zoff=None, accumulate=False, stream=None):
    torch = _torch()
    L = load()
    gc = _geom(g)
    nz = g.Z if nz is None else nz
    zoff = L.tk_default_zoff(ctypes.byref(gc)) if zoff is None else zoff
    if vol is None:
        vol = torch.empty((nz, g.Y, g.X), dtype=torch.float32, device=q.device)
    check(L.tk_backproject(ctypes.byref(gc), q.data_ptr(), precision,
                           None if scale is None else scale.data_ptr(), int(nz), float(zoff), vol.data_ptr(),
                           int(bool(accumulate)), _stream_ptr(stream)))
    return vol


def workspace_bytes(g, precision=_lib.TK_F32) -> int:
    gc = _geom(g)
    return int(load().tk_fdk_workspace_bytes(ctypes.byref(gc), precision))


def fdk_device(g, d_in, input_type=_lib.TK_INPUT_F32, layout=_lib.TK_LAYOUT_SINOGRAM, ff=None,
               window=_lib.TK_WINDOW_RAMLAK, precision=_lib.TK_F32, workspace=None, vol=None, stream=None):
    torch = _torch()
    L = load()
    gc = _geom(g)
    nb = workspace_bytes(g, precision)
    if workspace is None:
        workspace = torch.empty(nb, dtype=torch.uint8, device=d_in.device)
    if vol is None:
        vol = torch.empty((g.Z, g.Y, g.X), dtype=torch.float32, device=d_in.device)
    check(L.tk_fdk_device(ctypes.byref(gc), d_in.data_ptr(), input_type, layout,
                          None if ff is None else ctypes.byref(ff), window, precision, workspace.data_ptr(),
                          workspace.numel(), vol.data_ptr(), _stream_ptr(stream)))
    return vol


def stream_workspace_bytes(g, input_type=_lib.TK_INPUT_U16, precision=_lib.TK_F16, chunk=64) -> int:
    gc = _geom(g)
    return int(load().tk_fdk_stream_workspace_bytes(ctypes.byref(gc), input_type, precision, int(chunk)))


def fdk_stream(g, h_in, input_type=_lib.TK_INPUT_U16, ff=None, window=_lib.TK_WINDOW_RAMLAK,
               precision=_lib.TK_F16, chunk=64, workspace=None, vol=None, stream=None, device=None):
    """Out-of-core FDK: h_in is a host (preferably pinned) tensor or array of
    projection-major [N][H][W] data, streamed to the GPU in chunks."""
    torch = _torch()
    L = load()
    gc = _geom(g)
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    if workspace is None:
        workspace = torch.empty(stream_workspace_bytes(g, input_type, precision, chunk), dtype=torch.uint8,
                                device=dev)
    if vol is None:
        vol = torch.empty((g.Z, g.Y, g.X), dtype=torch.float32, device=dev)
    ptr = h_in.data_ptr() if hasattr(h_in, "data_ptr") else h_in.ctypes.data
    check(L.tk_fdk_stream(ctypes.byref(gc), ptr, input_type, None if ff is None else ctypes.byref(ff), window,
                          precision, int(chunk), workspace.data_ptr(), workspace.numel(), vol.data_ptr(),
                          _stream_ptr(stream)))
    return vol


def half_to_full_fan(sino, axis_move: int, D: float, dfi: float, flip=False, out=None, stream=None):
    """Half-fan completion of fan-beam sinograms sino [rows][N][W] (device FP32)."""
    torch = _torch()
    rows, N, W = sino.shape
    if out is None:
        out = torch.empty((rows, N, 2 * W - 1 - 2 * axis_move), dtype=torch.float32, device=sino.device)
    check(load().tk_half_to_full_fan(sino.data_ptr(), W, N, rows, int(axis_move), float(D), float(dfi),
                                     int(bool(flip)), out.data_ptr(), _stream_ptr(stream)))
    return out


def half_to_parallel(sino, axis_move: int, D: float, dfi: float, out=None, stream=None):
    """Fan->parallel rebinning of half-fan sinograms sino [rows][N][W] (device FP32)."""
    torch = _torch()
    rows, N, W = sino.shape
    if out is None:
        out = torch.empty((rows, N // 2, 2 * W - 1 - 2 * axis_move), dtype=torch.float32, device=sino.device)
    check(load().tk_half_to_parallel(sino.data_ptr(), W, N, rows, int(axis_move), float(D), float(dfi),
                                     out.data_ptr(), _stream_ptr(stream)))
    return out


def forward_project(g, vol, nz=None, zoff=None, out=None, accumulate=False, stream=None):
    """B^T: transpose of the backprojection; returns [N][H][Wp] FP32."""
    torch = _torch()
    L = load()
    gc = _geom(g)
    nz = g.Z if nz is None else nz
    zoff = L.tk_default_zoff(ctypes.byref(gc)) if zoff is None else zoff
    if out is None:
        out = torch.empty((g.N, g.H, row_pitch(g.W)), dtype=torch.float32, device=vol.device)
    check(L.tk_forward_project(ctypes.byref(gc), vol.data_ptr(), int(nz), float(zoff), out.data_ptr(),
                               int(bool(accumulate)), _stream_ptr(stream)))
    return out


def filter_transpose(g, qbar, window=_lib.TK_WINDOW_RAMLAK, layout=_lib.TK_LAYOUT_SINOGRAM, out=None, stream=None):
    torch = _torch()
    L = load()
    gc = _geom(g)
    shape = (g.H, g.N, g.W) if layout == _lib.TK_LAYOUT_SINOGRAM else (g.N, g.H, g.W)
    if out is None:
        out = torch.empty(shape, dtype=torch.float32, device=qbar.device)
    check(L.tk_filter_transpose(ctypes.byref(gc), qbar.data_ptr(), window, out.data_ptr(), layout,
                                _stream_ptr(stream)))
    return out


def fdk_backward(g, vol_grad, window=_lib.TK_WINDOW_RAMLAK, layout=_lib.TK_LAYOUT_SINOGRAM, workspace=None,
                 out=None, stream=None):
    """A^T: gradient of a volume loss with respect to the line integrals."""
    torch = _torch()
    L = load()
    gc = _geom(g)
    nb = workspace_bytes(g, _lib.TK_F32)
    if workspace is None:
        workspace = torch.empty(nb, dtype=torch.uint8, device=vol_grad.device)
    shape = (g.H, g.N, g.W) if layout == _lib.TK_LAYOUT_SINOGRAM else (g.N, g.H, g.W)
    if out is None:
        out = torch.empty(shape, dtype=torch.float32, device=vol_grad.device)
    check(L.tk_fdk_backward(ctypes.byref(gc), vol_grad.data_ptr(), layout, window, workspace.data_ptr(),
                            workspace.numel(), out.data_ptr(), _stream_ptr(stream)))
    return out


def refine_workspace(g, device="cuda"):
    torch = _torch()
    return torch.empty(load().tk_refine_workspace_bytes(ctypes.byref(_geom(g))), dtype=torch.uint8, device=device)


def refine_checkpoint(g, d_in, input_type=_lib.TK_INPUT_F32, layout=_lib.TK_LAYOUT_SINOGRAM, ff=None,
                      window=_lib.TK_WINDOW_RAMLAK, precision=_lib.TK_F32, workspace=None, stream=None):
    """Filtered projections q = F W p checkpointed as FP32 or FP16 samples [N][H][Wp]."""
    torch = _torch()
    L = load()
    gc = _geom(g)
    dt = torch.float16 if precision == _lib.TK_F16 else torch.float32
    ckpt = torch.empty((g.N, g.H, row_pitch(g.W)), dtype=dt, device=d_in.device)
    ws = refine_workspace(g, d_in.device) if workspace is None else workspace
    check(L.tk_refine_checkpoint(ctypes.byref(gc), d_in.data_ptr(), input_type, layout,
                                 None if ff is None else ctypes.byref(ff), window, ckpt.data_ptr(), precision,
                                 ws.data_ptr(), ws.numel(), _stream_ptr(stream)))
    return ckpt


def refine_step_size(g, iters=6, vol_tmp=None, workspace=None, stream=None) -> float:
    """1 / lambda_max(B B^T) by power iteration (a step size that lowers the loss at every step)."""
    torch = _torch()
    L = load()
    gc = _geom(g)
    ws = refine_workspace(g) if workspace is None else workspace
    v = torch.empty((g.Z, g.Y, g.X), dtype=torch.float32, device=ws.device) if vol_tmp is None else vol_tmp
    a = ctypes.c_float(0.0)
    check(L.tk_refine_step_size(ctypes.byref(gc), int(iters), v.data_ptr(), ws.data_ptr(), ws.numel(),
                                ctypes.byref(a), _stream_ptr(stream)))
    return float(a.value)


def refine_volume(g, ckpt, vol, alpha, steps, loss=None, workspace=None, stream=None):
    """`steps` data-consistency steps on vol in place; loss (float64 device tensor of `steps`) gets L(x_k)."""
    L = load()
    gc = _geom(g)
    prec = _lib.TK_F16 if str(ckpt.dtype) == "torch.float16" else _lib.TK_F32
    ws = refine_workspace(g, vol.device) if workspace is None else workspace
    check(L.tk_refine_volume(ctypes.byref(gc), ckpt.data_ptr(), prec, float(alpha), int(steps), vol.data_ptr(),
                             None if loss is None else loss.data_ptr(), ws.data_ptr(), ws.numel(),
                             _stream_ptr(stream)))
    return vol


def phantom_project(g, ell: np.ndarray, layout=_lib.TK_LAYOUT_SINOGRAM, out=None, device="cuda", stream=None):
    """Analytic line integrals of ellipsoids on the GPU (FP32)."""
    torch = _torch()
    L = load()
    gc = _geom(g)
    e = np.ascontiguousarray(ell, dtype=np.float64).reshape(-1, 16)
    shape = (g.H, g.N, g.W) if layout == _lib.TK_LAYOUT_SINOGRAM else (g.N, g.H, g.W)
    if out is None:
        out = torch.empty(shape, dtype=torch.float32, device=device)
    check(L.tk_phantom_project(ctypes.byref(gc), e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), e.shape[0],
                               layout, out.data_ptr(), _stream_ptr(stream)))
    return out


def device_error_flags(clear=True) -> int:
    v = ctypes.c_uint()
    check(load().tk_device_error_flags(ctypes.byref(v), int(bool(clear))))
    return v.value
