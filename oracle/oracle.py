"""ctypes front end of the CPU oracle (oracle/tk_oracle.c).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by ``__graft_entry__.smoke()``
as the checker and by bench.py's CPU-baseline leg; the shipped package never
imports it.

The oracle restates the reference FDK (Lukas-kV/TomoKvas FBPG/kernel.cu):
``fdk_f32`` follows the reference's FP32 operation order (cosine weight
kernel.cu:179-201, FFT ramp filter kernel.cu:557-802, backprojection
kernel.cu:68-177); ``fdk_f64`` is the same discretisation in double.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libtk_oracle.so")
SOURCES = [os.path.join(HERE, "tk_oracle.c"), os.path.join(HERE, "tk_oracle.h")]

WIN_RAMLAK, WIN_SHEPP_LOGAN, WIN_HANN = 0, 1, 2
WINDOWS = {"ramlak": WIN_RAMLAK, "shepp_logan": WIN_SHEPP_LOGAN, "hann": WIN_HANN}


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (portable flags; no x86 or Arm specifics)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off",
           "-pthread", SOURCES[0], "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Geom(ctypes.Structure):
    """Mirror of ``orc_geom`` (reference parameter set, kernel.cu:479-537)."""

    _fields_ = [
        ("W", ctypes.c_int), ("N", ctypes.c_int), ("H", ctypes.c_int),
        ("cX", ctypes.c_float), ("cZ", ctypes.c_float), ("dfi", ctypes.c_float),
        ("D", ctypes.c_float), ("tau", ctypes.c_float),
        ("X", ctypes.c_int), ("Y", ctypes.c_int), ("Z", ctypes.c_int),
        ("cx", ctypes.c_float), ("cy", ctypes.c_float), ("cz", ctypes.c_float),
        ("rot", ctypes.c_float), ("scale", ctypes.c_float),
        ("dirx", ctypes.c_int), ("diry", ctypes.c_int), ("dirz", ctypes.c_int),
        ("zb", ctypes.c_int),
    ]


def geom_from(p) -> Geom:
    """Build a Geom from any object with the reference parameter attributes."""
    g = Geom()
    for name, _ in Geom._fields_:
        setattr(g, name, getattr(p, name))
    return g


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(build())
        _declare(_LIB)
    return _LIB


def _declare(L):
    P = ctypes.POINTER
    f32p, f64p, i32p = P(ctypes.c_float), P(ctypes.c_double), P(ctypes.c_int)
    gp = P(Geom)
    L.orc_pad_length.argtypes = [ctypes.c_int]
    L.orc_filter_kernel_f64.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, f64p]
    L.orc_zblocks.argtypes = [gp, f32p, ctypes.c_int]
    L.orc_weight_f32.argtypes = [f32p, gp]
    L.orc_filter_f32.argtypes = [f32p, f32p, gp, ctypes.c_int, ctypes.c_int]
    L.orc_bp_f32.argtypes = [f32p, gp, i32p, ctypes.c_int, f32p, ctypes.c_int]
    L.orc_fdk_f32.argtypes = [f32p, gp, ctypes.c_int, i32p, ctypes.c_int, f32p, ctypes.c_int]
    L.orc_weight_filter_f64.argtypes = [f32p, f64p, gp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.orc_bp_f64.argtypes = [f64p, gp, i32p, ctypes.c_int, f64p, ctypes.c_int, ctypes.c_int]
    L.orc_fdk_f64.argtypes = [f32p, gp, ctypes.c_int, i32p, ctypes.c_int, f64p, ctypes.c_int]
    L.orc_rows_needed.argtypes = [gp, i32p, ctypes.c_int, i32p, i32p]
    L.orc_fdk_adjoint_f64.argtypes = [f32p, gp, ctypes.c_int, f64p, ctypes.c_int]
    L.orc_b_f64.argtypes = [f64p, gp, f64p, ctypes.c_int]
    L.orc_bt_f64.argtypes = [f64p, gp, f64p, ctypes.c_int]
    d = ctypes.c_double
    L.orc_fdk_u16_f32_sampled.argtypes = [P(ctypes.c_uint16), d, d, d, d, ctypes.c_int, d, gp, ctypes.c_int,
                                          i32p, ctypes.c_int, f32p, ctypes.c_int]
    L.orc_fdk_u16_f64_sampled.argtypes = [P(ctypes.c_uint16), d, d, d, d, ctypes.c_int, d, gp, ctypes.c_int,
                                          i32p, ctypes.c_int, f64p, ctypes.c_int]
    L.orc_half2fullfan_f64.argtypes = [f64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, d, d,
                                       ctypes.c_int, f64p]
    L.orc_half2para_f64.argtypes = [f64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, d, d, f64p]
    L.orc_log_u16_f64.argtypes = [P(ctypes.c_uint16), f32p, f32p, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                  ctypes.c_double, f32p, ctypes.c_int]
    L.orc_project_ellipsoids.argtypes = [f64p, ctypes.c_int, gp, ctypes.c_int, f32p, ctypes.c_int]
    L.orc_voxelise_ellipsoids.argtypes = [f64p, ctypes.c_int, gp, i32p, ctypes.c_int, f32p, ctypes.c_int]


def _ptr(a: np.ndarray, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def _threads(n):
    return n if n else (os.cpu_count() or 1)


def _zlist(g: Geom, zlist):
    z = np.arange(g.Z, dtype=np.int32) if zlist is None else np.ascontiguousarray(zlist, dtype=np.int32)
    return z


def pad_length(W: int) -> int:
    return lib().orc_pad_length(W)


def filter_kernel(W: int, tau: float, window="ramlak", p: int = 0):
    """Effective spatial kernel k[n], n = -(W-1)..W-1 (index n + W - 1), and p."""
    k = np.zeros(2 * W - 1, dtype=np.float64)
    win = WINDOWS[window] if isinstance(window, str) else int(window)
    pp = lib().orc_filter_kernel_f64(W, tau, win, p, _ptr(k, ctypes.c_double))
    if pp < 0:
        raise ValueError("bad filter arguments")
    return k, pp


def zblocks(g: Geom):
    buf = np.zeros(65536, dtype=np.float32)
    n = lib().orc_zblocks(ctypes.byref(g), _ptr(buf, ctypes.c_float), 65536)
    return buf[:n].copy()


def weight_f32(sino: np.ndarray, g: Geom) -> np.ndarray:
    s = np.ascontiguousarray(sino, dtype=np.float32).copy()
    lib().orc_weight_f32(_ptr(s, ctypes.c_float), ctypes.byref(g))
    return s


def filter_f32(weighted: np.ndarray, g: Geom, window="ramlak", nthreads=0) -> np.ndarray:
    w = np.ascontiguousarray(weighted, dtype=np.float32)
    q = np.empty_like(w)
    win = WINDOWS[window] if isinstance(window, str) else int(window)
    lib().orc_filter_f32(_ptr(w, ctypes.c_float), _ptr(q, ctypes.c_float), ctypes.byref(g), win, _threads(nthreads))
    return q


def bp_f32(q: np.ndarray, g: Geom, zlist=None, nthreads=0) -> np.ndarray:
    qq = np.ascontiguousarray(q, dtype=np.float32)
    z = _zlist(g, zlist)
    vol = np.zeros((len(z), g.Y, g.X), dtype=np.float32)
    lib().orc_bp_f32(_ptr(qq, ctypes.c_float), ctypes.byref(g), _ptr(z, ctypes.c_int), len(z),
                     _ptr(vol, ctypes.c_float), _threads(nthreads))
    return vol


def fdk_f32(sino: np.ndarray, g: Geom, window="ramlak", zlist=None, nthreads=0) -> np.ndarray:
    """FP32 restatement of the reference FDK; sino is [H][N][W]."""
    s = np.ascontiguousarray(sino, dtype=np.float32)
    assert s.shape == (g.H, g.N, g.W), s.shape
    z = _zlist(g, zlist)
    vol = np.zeros((len(z), g.Y, g.X), dtype=np.float32)
    win = WINDOWS[window] if isinstance(window, str) else int(window)
    rc = lib().orc_fdk_f32(_ptr(s, ctypes.c_float), ctypes.byref(g), win, _ptr(z, ctypes.c_int), len(z),
                           _ptr(vol, ctypes.c_float), _threads(nthreads))
    if rc:
        raise MemoryError("oracle fdk_f32 failed")
    return vol


def fdk_u16_f32_sampled(raw: np.ndarray, g: Geom, flat: float, dark: float = 0.0, A=1.0, B=0.0, invert=True,
                        floor_counts=0.5, window="ramlak", zlist=None, nthreads=0) -> np.ndarray:
    """FP32 restatement from raw uint16 [N][H][W] on sampled slices (CPU baseline)."""
    r = np.ascontiguousarray(raw).view(np.uint16)
    assert r.shape == (g.N, g.H, g.W), r.shape
    z = _zlist(g, zlist)
    vol = np.zeros((len(z), g.Y, g.X), dtype=np.float32)
    win = WINDOWS[window] if isinstance(window, str) else int(window)
    rc = lib().orc_fdk_u16_f32_sampled(_ptr(r, ctypes.c_uint16), dark, flat, A, B, int(bool(invert)), floor_counts,
                                       ctypes.byref(g), win, _ptr(z, ctypes.c_int), len(z),
                                       _ptr(vol, ctypes.c_float), _threads(nthreads))
    if rc:
        raise MemoryError("oracle fdk_u16_f32_sampled failed")
    return vol


def fdk_u16_f64_sampled(raw: np.ndarray, g: Geom, flat: float, dark: float = 0.0, A=1.0, B=0.0, invert=True,
                        floor_counts=0.5, window="ramlak", zlist=None, nthreads=0) -> np.ndarray:
    """FP64 oracle from raw uint16 [N][H][W] on sampled slices, streaming the
    projections in small blocks (memory independent of N)."""
    r = np.ascontiguousarray(raw).view(np.uint16)
    assert r.shape == (g.N, g.H, g.W), r.shape
    z = _zlist(g, zlist)
    vol = np.zeros((len(z), g.Y, g.X), dtype=np.float64)
    win = WINDOWS[window] if isinstance(window, str) else int(window)
    rc = lib().orc_fdk_u16_f64_sampled(_ptr(r, ctypes.c_uint16), dark, flat, A, B, int(bool(invert)), floor_counts,
                                       ctypes.byref(g), win, _ptr(z, ctypes.c_int), len(z),
                                       _ptr(vol, ctypes.c_double), _threads(nthreads))
    if rc:
        raise MemoryError("oracle fdk_u16_f64_sampled failed")
    return vol


def half2fullfan(sino: np.ndarray, axis_move: int, D: float, dfi: float, flip=False) -> np.ndarray:
    """Half-fan completion of sinograms [rows][N][W] (double)."""
    x = np.ascontiguousarray(sino, dtype=np.float64)
    rows, N, W = x.shape
    out = np.empty((rows, N, 2 * W - 1 - 2 * axis_move), dtype=np.float64)
    lib().orc_half2fullfan_f64(_ptr(x, ctypes.c_double), W, N, rows, axis_move, D, dfi, int(bool(flip)),
                               _ptr(out, ctypes.c_double))
    return out


def half2para(sino: np.ndarray, axis_move: int, D: float, dfi: float) -> np.ndarray:
    """Fan->parallel rebinning of half-fan sinograms [rows][N][W] (double)."""
    x = np.ascontiguousarray(sino, dtype=np.float64)
    rows, N, W = x.shape
    out = np.empty((rows, N // 2, 2 * W - 1 - 2 * axis_move), dtype=np.float64)
    lib().orc_half2para_f64(_ptr(x, ctypes.c_double), W, N, rows, axis_move, D, dfi, _ptr(out, ctypes.c_double))
    return out


def fdk_adjoint_f64(vol: np.ndarray, g: Geom, window="ramlak", nthreads=0) -> np.ndarray:
    """FP64 transpose of the FDK (volume [Z][Y][X] -> line-integral gradient [H][N][W])."""
    v = np.ascontiguousarray(vol, dtype=np.float32)
    assert v.shape == (g.Z, g.Y, g.X), v.shape
    out = np.empty((g.H, g.N, g.W), dtype=np.float64)
    win = WINDOWS[window] if isinstance(window, str) else int(window)
    if lib().orc_fdk_adjoint_f64(_ptr(v, ctypes.c_float), ctypes.byref(g), win, _ptr(out, ctypes.c_double),
                                 _threads(nthreads)):
        raise MemoryError("oracle adjoint failed")
    return out


def b_f64(q: np.ndarray, g: Geom, nthreads=0) -> np.ndarray:
    """FP64 plain backprojection B of q [N][H][W] (scale dfi/p), volume [Z][Y][X]."""
    x = np.ascontiguousarray(q, dtype=np.float64)
    assert x.shape == (g.N, g.H, g.W), x.shape
    out = np.empty((g.Z, g.Y, g.X), dtype=np.float64)
    if lib().orc_b_f64(_ptr(x, ctypes.c_double), ctypes.byref(g), _ptr(out, ctypes.c_double), _threads(nthreads)):
        raise MemoryError("oracle backprojection failed")
    return out


def bt_f64(vol: np.ndarray, g: Geom, nthreads=0) -> np.ndarray:
    """FP64 transpose B^T of the plain backprojection: volume [Z][Y][X] -> q [N][H][W]."""
    v = np.ascontiguousarray(vol, dtype=np.float64)
    assert v.shape == (g.Z, g.Y, g.X), v.shape
    out = np.empty((g.N, g.H, g.W), dtype=np.float64)
    if lib().orc_bt_f64(_ptr(v, ctypes.c_double), ctypes.byref(g), _ptr(out, ctypes.c_double), _threads(nthreads)):
        raise MemoryError("oracle forward projection failed")
    return out


def rows_needed(g: Geom, zlist):
    z = _zlist(g, zlist)
    lo, hi = ctypes.c_int(), ctypes.c_int()
    lib().orc_rows_needed(ctypes.byref(g), _ptr(z, ctypes.c_int), len(z), ctypes.byref(lo), ctypes.byref(hi))
    return lo.value, hi.value


def weight_filter_f64(sino: np.ndarray, g: Geom, window="ramlak", rows=None, nthreads=0) -> np.ndarray:
    s = np.ascontiguousarray(sino, dtype=np.float32)
    lo, hi = (0, g.H - 1) if rows is None else rows
    q = np.empty((hi - lo + 1, g.N, g.W), dtype=np.float64)
    win = WINDOWS[window] if isinstance(window, str) else int(window)
    lib().orc_weight_filter_f64(_ptr(s, ctypes.c_float), _ptr(q, ctypes.c_double), ctypes.byref(g), win,
                                lo, hi, _threads(nthreads))
    return q


def fdk_f64(sino: np.ndarray, g: Geom, window="ramlak", zlist=None, nthreads=0) -> np.ndarray:
    """FP64 FDK oracle; sino is [H][N][W].  Only the rows the slices need are filtered."""
    s = np.ascontiguousarray(sino, dtype=np.float32)
    assert s.shape == (g.H, g.N, g.W), s.shape
    z = _zlist(g, zlist)
    vol = np.zeros((len(z), g.Y, g.X), dtype=np.float64)
    win = WINDOWS[window] if isinstance(window, str) else int(window)
    rc = lib().orc_fdk_f64(_ptr(s, ctypes.c_float), ctypes.byref(g), win, _ptr(z, ctypes.c_int), len(z),
                           _ptr(vol, ctypes.c_double), _threads(nthreads))
    if rc:
        raise MemoryError("oracle fdk_f64 failed")
    return vol


def log_u16(raw: np.ndarray, flat: np.ndarray, dark=None, A=1.0, B=0.0, invert=True,
            floor_counts=0.5, nthreads=0) -> np.ndarray:
    """Flat-field + log (rsq_load.cpp:299-325); raw [N][H][W] -> sinogram [H][N][W]."""
    r = np.ascontiguousarray(raw, dtype=np.uint16)
    N, H, W = r.shape
    fl = np.ascontiguousarray(np.broadcast_to(flat, (H, W)), dtype=np.float32)
    dk = None if dark is None else np.ascontiguousarray(np.broadcast_to(dark, (H, W)), dtype=np.float32)
    out = np.empty((H, N, W), dtype=np.float32)
    lib().orc_log_u16_f64(_ptr(r, ctypes.c_uint16), None if dk is None else _ptr(dk, ctypes.c_float),
                          _ptr(fl, ctypes.c_float), W, N, H, A, B, int(bool(invert)), floor_counts,
                          _ptr(out, ctypes.c_float), _threads(nthreads))
    return out


def project_ellipsoids(ell: np.ndarray, g: Geom, layout="sino", nthreads=0) -> np.ndarray:
    """Analytic line integrals; layout 'sino' -> [H][N][W], 'proj' -> [N][H][W]."""
    e = np.ascontiguousarray(ell, dtype=np.float64).reshape(-1, 16)
    lay = 0 if layout == "sino" else 1
    shape = (g.H, g.N, g.W) if lay == 0 else (g.N, g.H, g.W)
    out = np.empty(shape, dtype=np.float32)
    lib().orc_project_ellipsoids(_ptr(e, ctypes.c_double), e.shape[0], ctypes.byref(g), lay,
                                 _ptr(out, ctypes.c_float), _threads(nthreads))
    return out


def voxelise_ellipsoids(ell: np.ndarray, g: Geom, zlist=None, nthreads=0) -> np.ndarray:
    e = np.ascontiguousarray(ell, dtype=np.float64).reshape(-1, 16)
    z = _zlist(g, zlist)
    vol = np.zeros((len(z), g.Y, g.X), dtype=np.float32)
    lib().orc_voxelise_ellipsoids(_ptr(e, ctypes.c_double), e.shape[0], ctypes.byref(g), _ptr(z, ctypes.c_int),
                                  len(z), _ptr(vol, ctypes.c_float), _threads(nthreads))
    return vol
