"""Python mirror of the reference engine class FilteredBackProjection.

Same method names, argument order, units and call sequence as
Lukas-kV/TomoKvas FBPG/kernel.cuh:82-151 (driven as in FBPG/para_TC.cpp:130-153);
every call goes straight to libtk_fdk.so through its C ABI.  Methods return
the status code like the reference returns cudaError_t (0 = success) and
``last_error()`` gives the message; ``raise_on_error=True`` raises instead.

The output object passed to ``SetReconstructionProperties`` plays the role of
the reference's ``bin_siz``: it must provide ``GetBlock(n, collecting)``
returning a C-contiguous float32 numpy buffer of at least X*Y*ZB elements
(FBPG/mucat_file.cpp:576-642).  ``VolumeSink`` is an in-memory implementation.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check, load


class VolumeSink:
    """In-memory bin_siz: hands out consecutive Z slabs of one [Z][Y][X] volume.

    With collecting (angle blocks accumulated over several engine runs) the
    slab already holds the previous partial sum, as the reference's READ
    prefetch provides (FBPG/mucat_file.cpp:610-624)."""

    def __init__(self, X: int, Y: int, Z: int, zb: int, out: np.ndarray | None = None):
        self.X, self.Y, self.Z, self.zb = X, Y, Z, zb
        self.volume = np.zeros((Z, Y, X), dtype=np.float32) if out is None else out
        assert self.volume.shape == (Z, Y, X) and self.volume.dtype == np.float32
        assert self.volume.flags.c_contiguous
        self.blocks_requested = []

    def GetBlock(self, n: int, collecting: bool = False) -> np.ndarray:
        self.blocks_requested.append((n, bool(collecting)))
        z0 = n * self.zb
        return self.volume[z0:z0 + self.zb]


class FilteredBackProjection:
    def __init__(self, raise_on_error: bool = False):
        self._L = load()
        h = ctypes.c_void_p()
        check(self._L.tk_fdk_create(ctypes.byref(h)))
        self._h = h
        self._raise = raise_on_error
        self._keep = []  # host arrays borrowed until Initialize returns
        self._out = None
        self._blocks = {}
        self._zb = 16

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.tk_fdk_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _rc(self, rc: int) -> int:
        if rc != 0 and self._raise:
            check(rc)
        return rc

    @staticmethod
    def last_error() -> str:
        return load().tk_last_error().decode(errors="replace")

    # -- reference setters (kernel.cuh:89-108) ----------------------------
    def SetGPUid(self, gpu_id: int = 0):
        return self._rc(self._L.tk_fdk_set_gpu_id(self._h, int(gpu_id)))

    def SetBlockSize(self, sz: int = 16):
        self._zb = int(sz)
        return self._rc(self._L.tk_fdk_set_block_size(self._h, int(sz)))

    def SetAllocationLimit(self, memory_limit: int = 1024 ** 3):
        return self._rc(self._L.tk_fdk_set_allocation_limit(self._h, int(memory_limit)))

    def SetCollecting(self, collecting: bool = False):
        return self._rc(self._L.tk_fdk_set_collecting(self._h, int(bool(collecting))))

    def SetShowInfo(self, show: bool = False):
        return self._rc(self._L.tk_fdk_set_show_info(self._h, int(bool(show))))

    def SetAxisDirection(self, X: bool = False, Y: bool = False, Z: bool = False):
        return self._rc(self._L.tk_fdk_set_axis_direction(self._h, int(bool(X)), int(bool(Y)), int(bool(Z))))

    def SetSinogramProperties(self, sinogram, sinogram_X, centre_X, sinogram_Y, sinogram_Z, centre_Z,
                              delta_fi, distance, sampling):
        """sinogram: float32 [sin_Z][sin_Y][sin_X] (rows, angles, columns), or None
        when the projections come from SetProjectionsU16."""
        ptr = None
        if sinogram is not None:
            s = np.ascontiguousarray(sinogram, dtype=np.float32)
            assert s.size == int(sinogram_X) * int(sinogram_Y) * int(sinogram_Z)
            self._keep.append(s)
            ptr = s.ctypes.data
        return self._rc(self._L.tk_fdk_set_sinogram_properties(
            self._h, ptr, int(sinogram_X), float(centre_X), int(sinogram_Y), int(sinogram_Z), float(centre_Z),
            float(delta_fi), float(distance), float(sampling)))

    def SetReconstructionProperties(self, output_file, reconstruction_X, centre_X, reconstruction_Y, centre_Y,
                                    reconstruction_Z, centre_Z, rot):
        self._out = output_file
        return self._rc(self._L.tk_fdk_set_reconstruction_properties(
            self._h, int(reconstruction_X), float(centre_X), int(reconstruction_Y), float(centre_Y),
            int(reconstruction_Z), float(centre_Z), float(rot)))

    def SetScaleXYZ(self, scale: float):
        return self._rc(self._L.tk_fdk_set_scale_xyz(self._h, float(scale)))

    def Initialize(self) -> int:
        rc = self._rc(self._L.tk_fdk_initialize(self._h))
        self._keep.clear()  # borrowed host data may be released now (para_TC.cpp:150)
        return rc

    def CalculateReconstruction(self) -> int:
        if self._out is None:
            raise RuntimeError("SetReconstructionProperties needs an output object with GetBlock")
        out = self._out
        live = {}

        def sink(_user, n, collecting):
            try:
                buf = out.GetBlock(int(n), bool(collecting))
                arr = np.asarray(buf)
                if arr.dtype != np.float32 or not arr.flags.c_contiguous:
                    return None
                live[n & 1] = arr  # keep alive while the engine writes into it
                return arr.ctypes.data
            except Exception:
                return None

        cb = _lib.BLOCK_SINK(sink)
        return self._rc(self._L.tk_fdk_calculate_reconstruction(self._h, cb, None))

    @staticmethod
    def GetFreeMemInfo(gpu_id: int) -> int:
        return int(load().tk_get_free_mem_info(int(gpu_id)))

    # -- extensions -------------------------------------------------------
    def SetProjectionsU16(self, raw, layout="projection", dark=None, flat=None, dark_value=0.0,
                          flat_value=0.0, A=1.0, B=0.0, invert=True, floor_counts=0.5):
        """Raw uint16 intensities; the log transform runs on the GPU.
        dark/flat: per-pixel [H][W] float arrays or None for the scalar values."""
        r = np.ascontiguousarray(raw, dtype=np.uint16)
        d = None if dark is None else np.ascontiguousarray(dark, dtype=np.float32)
        f = None if flat is None else np.ascontiguousarray(flat, dtype=np.float32)
        self._keep += [x for x in (r, d, f) if x is not None]
        return self._rc(self._L.tk_fdk_set_projections_u16(
            self._h, r.ctypes.data, _lib.LAYOUTS[layout], None if d is None else d.ctypes.data,
            None if f is None else f.ctypes.data, float(dark_value), float(flat_value), float(A), float(B),
            int(bool(invert)), float(floor_counts)))

    def SetInputLayout(self, layout: str):
        return self._rc(self._L.tk_fdk_set_input_layout(self._h, _lib.LAYOUTS[layout]))

    def SetFilter(self, window: str):
        return self._rc(self._L.tk_fdk_set_filter(self._h, _lib.WINDOWS[window]))

    def SetPrecision(self, precision: str):
        return self._rc(self._L.tk_fdk_set_precision(self._h, _lib.PRECISIONS[precision]))

    def SetPipeline(self, on: bool = True):
        """Reconstruct during Initialize, chunk by chunk as the projections upload (tk_fdk_set_pipeline)."""
        return self._rc(self._L.tk_fdk_set_pipeline(self._h, int(bool(on))))

    def SetStream(self, stream_handle: int):
        return self._rc(self._L.tk_fdk_set_stream(self._h, ctypes.c_void_p(stream_handle)))

    def ReconstructToDevice(self, device_ptr: int) -> int:
        """Whole volume into device memory at device_ptr ([Z][Y][X] float32)."""
        return self._rc(self._L.tk_fdk_reconstruct_device(self._h, ctypes.c_void_p(device_ptr)))

    def Timings(self) -> dict:
        vals = [ctypes.c_float() for _ in range(4)]
        check(self._L.tk_fdk_get_timings(self._h, *[ctypes.byref(v) for v in vals]))
        return dict(zip(("filter_ms", "bp_ms", "h2d_ms", "d2h_ms"), (v.value for v in vals)))
