"""C ABI surface, checked without a GPU: exports, host-only entry points, errors.

No call here launches a kernel or touches device memory.
"""
import ctypes
import os
import re

import numpy as np
import pytest

from _util import small_geometry
from tomokvas_gb300 import _lib
from tomokvas_gb300.geometry import FDKGeometry, config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(tk_[a-z0-9_]+)\s*\(", text))
    return names


def test_header_matches_binding_list():
    assert header_functions() == set(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(tklib):
    missing = [n for n in header_functions() if not hasattr(tklib, n)]
    assert not missing, missing


def test_version_and_pad_length(tklib):
    assert tklib.tk_version() == 1
    for W, p in [(1, 4), (256, 512), (1000, 2048), (1024, 2048), (2048, 4096)]:
        assert tklib.tk_pad_length(W) == p
    assert tklib.tk_pad_length(0) < 0


def test_zblock_offsets_match_oracle(tklib, orc):
    for Z, zb in [(256, 16), (255, 30), (1024, 30), (33, 16), (1, 16)]:
        g = small_geometry(vol=(8, 8, Z), zb=zb)
        gc = g.to_c()
        n = tklib.tk_zblock_offsets(ctypes.byref(gc), zb, None, 0)
        buf = (ctypes.c_float * max(n, 1))()
        assert tklib.tk_zblock_offsets(ctypes.byref(gc), zb, buf, n) == n
        exp = orc.zblocks(orc.geom_from(g))
        assert n == len(exp)
        assert np.array_equal(np.array(buf[:n], dtype=np.float32), exp)


def test_default_zoff(tklib):
    g = small_geometry(vol=(8, 8, 256))
    assert tklib.tk_default_zoff(ctypes.byref(g.to_c())) == -127.5


@pytest.mark.parametrize("field,value", [("W", 0), ("D", 0.0), ("tau", -1.0), ("scale", 0.0), ("X", 0),
                                         ("W", 5000), ("D", float("nan"))])
def test_invalid_geometry_rejected_before_any_device_work(tklib, field, value):
    g = small_geometry()
    gc = g.to_c()
    setattr(gc, field, value)
    rc = tklib.tk_backproject(ctypes.byref(gc), ctypes.c_void_p(16), 0, None, 8, 0.0, ctypes.c_void_p(16), 0, None)
    assert rc in (_lib.TK_ERR_INVALID, _lib.TK_ERR_UNSUPPORTED)
    assert tklib.tk_last_error()
    rc = tklib.tk_filter_projections(ctypes.byref(gc), ctypes.c_void_p(16), 0, 0, None, 0, ctypes.c_void_p(16), 0,
                                     None, None)
    assert rc in (_lib.TK_ERR_INVALID, _lib.TK_ERR_UNSUPPORTED)


def test_stage_argument_checks(tklib):
    g = small_geometry().to_c()
    # null device pointers
    assert tklib.tk_backproject(ctypes.byref(g), None, 0, None, 8, 0.0, None, 0, None) == _lib.TK_ERR_INVALID
    # 16-bit storage without its scale
    assert tklib.tk_backproject(ctypes.byref(g), ctypes.c_void_p(256), 1, None, 8, 0.0, ctypes.c_void_p(256), 0,
                                None) == _lib.TK_ERR_INVALID
    assert b"scale" in tklib.tk_last_error()
    # raw input without flat-field parameters
    assert tklib.tk_filter_projections(ctypes.byref(g), ctypes.c_void_p(256), 1, 0, None, 0, ctypes.c_void_p(256),
                                       0, None, None) == _lib.TK_ERR_INVALID
    # workspace too small
    assert tklib.tk_fdk_device(ctypes.byref(g), ctypes.c_void_p(256), 0, 0, None, 0, 0, ctypes.c_void_p(256), 16,
                               ctypes.c_void_p(256), None) == _lib.TK_ERR_INVALID


def test_workspace_bytes(tklib):
    g = small_geometry(W=60, N=10, H=7)
    gc = g.to_c()
    assert tklib.tk_fdk_workspace_bytes(ctypes.byref(gc), 0) == 256 + 10 * 7 * 64 * 4   # FP32 samples
    assert tklib.tk_fdk_workspace_bytes(ctypes.byref(gc), 1) == 256 + 10 * 7 * 60 * 8   # FP16 coefficients
    assert tklib.tk_fdk_workspace_bytes(ctypes.byref(gc), 2) == 256 + 10 * 7 * 60 * 8   # BF16 coefficients
    assert tklib.tk_fdk_workspace_bytes(ctypes.byref(gc), 3) == 256 + 10 * 7 * 60 * 16  # FP32 coefficients
    assert tklib.tk_fdk_workspace_bytes(ctypes.byref(gc), 4) == 0
    g2 = small_geometry(W=61, N=3, H=5).to_c()
    assert tklib.tk_filtered_bytes(ctypes.byref(g2), 1) == 3 * 5 * 62 * 8


def test_stream_workspace_and_argument_checks(tklib):
    g = small_geometry(W=60, N=10, H=7)
    gc = g.to_c()
    a = lambda x: (x + 255) // 256 * 256
    # header + two raw chunks + one filtered chunk, each 256-byte aligned
    assert tklib.tk_fdk_stream_workspace_bytes(ctypes.byref(gc), 1, 1, 4) == 256 + 2 * a(4 * 7 * 60 * 2) + a(
        4 * 7 * 60 * 8)
    assert tklib.tk_fdk_stream_workspace_bytes(ctypes.byref(gc), 0, 0, 64) == 256 + 2 * a(10 * 7 * 60 * 4) + a(
        10 * 7 * 64 * 4)
    assert tklib.tk_fdk_stream_workspace_bytes(ctypes.byref(gc), 0, 0, 0) == 0
    assert tklib.tk_fdk_stream_workspace_bytes(ctypes.byref(gc), 5, 0, 4) == 0
    p = ctypes.c_void_p(256)
    # chunk 0, null host input, workspace too small: rejected before any device work
    assert tklib.tk_fdk_stream(ctypes.byref(gc), p, 0, None, 0, 0, 0, p, 1 << 20, p, None) == _lib.TK_ERR_INVALID
    assert tklib.tk_fdk_stream(ctypes.byref(gc), None, 0, None, 0, 0, 4, p, 1 << 20, p, None) == _lib.TK_ERR_INVALID
    assert tklib.tk_fdk_stream(ctypes.byref(gc), p, 0, None, 0, 0, 4, p, 16, p, None) == _lib.TK_ERR_INVALID
    assert b"workspace" in tklib.tk_last_error()


def test_rebin_argument_checks(tklib):
    import math

    p = ctypes.c_void_p(256)
    # rotation axis beyond the detector; not a full 360-degree scan; odd angle count for parallel rebinning
    assert tklib.tk_half_to_full_fan(p, 8, 10, 1, 7, 100.0, 2 * math.pi / 10, 0, p, None) == _lib.TK_ERR_INVALID
    assert tklib.tk_half_to_parallel(p, 8, 10, 1, 2, 100.0, 0.1, p, None) == _lib.TK_ERR_UNSUPPORTED
    assert tklib.tk_half_to_parallel(p, 8, 9, 1, 2, 100.0, 2 * math.pi / 9, p, None) == _lib.TK_ERR_INVALID
    assert tklib.tk_half_to_full_fan(p, 8, 10, 1, 2, 5.0, 2 * math.pi / 10, 0, p, None) == _lib.TK_ERR_INVALID


def test_diagnostics_without_gpu(tklib):
    assert tklib.tk_kernel_launches() >= 0
    assert tklib.tk_measure_fp32_fma_rate(None) == _lib.TK_ERR_INVALID


def test_handle_setters_and_state_errors(tklib):
    from tomokvas_gb300 import FilteredBackProjection

    fbp = FilteredBackProjection()
    assert fbp.SetGPUid(0) == 0
    assert fbp.SetBlockSize(30) == 0
    assert fbp.SetBlockSize(0) == _lib.TK_ERR_INVALID
    assert fbp.SetAllocationLimit(1 << 30) == 0
    assert fbp.SetCollecting(False) == 0
    assert fbp.SetAxisDirection(False, True, False) == 0
    assert fbp.SetFilter("hann") == 0
    assert fbp.SetPrecision("f16") == 0
    # Initialize before the properties are set is a sequencing error, not a crash
    assert fbp.Initialize() == _lib.TK_ERR_STATE
    assert "initialize" in fbp.last_error()
    fbp.close()


def test_geometry_mapping_of_workloads():
    c1 = config("c1")
    assert (c1.W, c1.N, c1.H, c1.X) == (256, 180, 256, 256)
    assert abs(c1.D - 2500.0) < 1e-9 and abs(c1.tau - 0.02) < 1e-12 and abs(c1.scale - 1.0) < 1e-12
    c2 = config("c2")
    assert abs(c2.D - 6000.0) < 1e-9 and abs(c2.tau - 0.005) < 1e-12 and abs(c2.scale - 1.0) < 1e-12
    assert c2.updates == 1024 ** 3 * 720
    c4 = config("c4")
    assert abs(c4.scale - 1.5) < 1e-12
    assert abs(config("c5").D - 12000.0) < 1e-6
    assert isinstance(c2, FDKGeometry)


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError, match="missing"):
        _lib._LIB_saved = _lib._LIB
        try:
            _lib._LIB = None
            _lib.load(str(tmp_path / "nope.so"))
        finally:
            _lib._LIB = _lib._LIB_saved
