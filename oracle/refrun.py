"""Runs the reference's own FDK kernels (see oracle/ref_build.py).

TEST INFRASTRUCTURE ONLY: generates the golden fixtures that pin the oracle.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import ref_build

_L = None


def lib():
    global _L
    if _L is None:
        L = ctypes.CDLL(ref_build.build_loader())
        f, i = ctypes.c_float, ctypes.c_int
        L.tkref_fdk.argtypes = [ctypes.c_char_p, ctypes.c_void_p, i, f, i, i, f, f, f, f, i, f, i, f, i, f, f, f,
                                i, i, i, i, ctypes.c_void_p, ctypes.c_void_p]
        L.tkref_last_error.restype = ctypes.c_char_p
        _L = L
    return _L


TIMES = ("upload_ms", "weight_ms", "filter_ms", "bp_kernels_ms", "reconstruction_ms", "total_ms")


def fdk(sino: np.ndarray, g, times: dict | None = None) -> np.ndarray:
    """Reference FDK of sinogram [H][N][W] with geometry g; returns [Z][Y][X].
    With `times`, fills the reference's stage times (see tkref_fdk)."""
    fatbin = ref_build.build_fatbin()
    if fatbin is None:
        raise RuntimeError("reference kernels not built: oracle/_ref/tk_ref_kernels.fatbin is missing")
    s = np.ascontiguousarray(sino, dtype=np.float32)
    vol = np.zeros((g.Z, g.Y, g.X), dtype=np.float32)
    t = np.zeros(6, dtype=np.float32)
    rc = lib().tkref_fdk(fatbin.encode(), s.ctypes.data, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau, g.X, g.cx,
                         g.Y, g.cy, g.Z, g.cz, g.rot, g.scale, g.dirx, g.diry, g.dirz, g.zb, vol.ctypes.data,
                         t.ctypes.data)
    if rc != 0:
        raise RuntimeError("reference run failed: " + lib().tkref_last_error().decode())
    if times is not None:
        times.update({k: float(v) for k, v in zip(TIMES, t)})
    return vol
