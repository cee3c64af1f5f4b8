"""Batches of uneven reconstructions: the tk_batch_* C ABI.

All items of a Batch are filtered (one launch each) and backprojected by one
persistent kernel launch; ``run(graph=True)`` replays a captured CUDA graph.
Device tensors passed to ``submit`` are referenced by the batch and must stay
allocated (they are kept alive here) and in place between runs.
"""
from __future__ import annotations

import ctypes

from . import _lib
from ._lib import check, load
from .device import _geom, _stream_ptr


class Batch:
    def __init__(self, precision=_lib.TK_F16):
        self._L = load()
        self._h = ctypes.c_void_p()
        check(self._L.tk_batch_create(ctypes.byref(self._h)))
        check(self._L.tk_batch_set_precision(self._h, precision))
        self._keep = []
        self.workspace = None

    def submit(self, g, d_in, vol, input_type=_lib.TK_INPUT_F32, layout=_lib.TK_LAYOUT_SINOGRAM, ff=None,
               window=_lib.TK_WINDOW_RAMLAK) -> int:
        gc = _geom(g)
        check(self._L.tk_batch_submit(self._h, ctypes.byref(gc), d_in.data_ptr(), input_type, layout,
                                      None if ff is None else ctypes.byref(ff), window, vol.data_ptr()))
        self._keep.append((d_in, vol, ff))
        return len(self) - 1

    def __len__(self):
        return int(self._L.tk_batch_size(self._h))

    def workspace_bytes(self) -> int:
        return int(self._L.tk_batch_workspace_bytes(self._h))

    def plan(self, workspace=None, stream=None):
        import torch

        nb = self.workspace_bytes()
        if workspace is None:
            workspace = torch.empty(nb, dtype=torch.uint8, device="cuda")
        self.workspace = workspace
        check(self._L.tk_batch_plan(self._h, workspace.data_ptr(), workspace.numel(), _stream_ptr(stream)))

    def run(self, graph=True, stream=None):
        check(self._L.tk_batch_run(self._h, int(bool(graph)), _stream_ptr(stream)))

    def autotune(self, stream=None):
        """Times each tile shape on this batch, keeps the fastest; returns (name, ms per run)."""
        v, ms = ctypes.c_int(-1), ctypes.c_float(0.0)
        check(self._L.tk_batch_autotune(self._h, _stream_ptr(stream), ctypes.byref(v), ctypes.byref(ms)))
        return self._L.tk_batch_variant_name(v.value).decode(), float(ms.value)

    def filter_forms(self) -> list:
        """Filter form of every item (TK_FILTER_*): what tk_batch_autotune chose by timing."""
        return [int(self._L.tk_batch_item_filter_form(self._h, i)) for i in range(self._L.tk_batch_size(self._h))]

    def quarter_turn_items(self) -> list:
        """Per item: True where the planned batch backprojects it with tk_fdk_device's quarter-turn launch."""
        return [int(self._L.tk_batch_item_quarter_turn(self._h, i)) == 1
                for i in range(self._L.tk_batch_size(self._h))]

    def timings(self):
        """(filter phase ms, backprojection ms) of the last eager run."""
        f, b = ctypes.c_float(0.0), ctypes.c_float(0.0)
        check(self._L.tk_batch_timings(self._h, ctypes.byref(f), ctypes.byref(b)))
        return float(f.value), float(b.value)

    def select_variant(self, i: int):
        check(self._L.tk_batch_select_variant(self._h, int(i)))

    @property
    def variant(self) -> str:
        return self._L.tk_batch_variant_name(self._L.tk_batch_variant(self._h)).decode()

    def close(self):
        if self._h:
            self._L.tk_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def variants(precision=None):
    """Names of the compiled batch tile shapes (optionally of one storage format)."""
    L = load()
    names = [L.tk_batch_variant_name(i).decode() for i in range(L.tk_batch_variant_count())]
    tag = {_lib.TK_F16: "<f16,", _lib.TK_BF16: "<bf16,", _lib.TK_F32_COEF: "<f32c,"}.get(precision)
    return [(i, n) for i, n in enumerate(names) if tag is None or tag in n]
