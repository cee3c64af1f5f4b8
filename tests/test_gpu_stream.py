"""Out-of-core FDK (tk_fdk_stream): projections streamed from host memory in
chunks while the volume accumulates in device memory.

Checks:
  * one chunk (chunk >= N) is bit-identical to the in-HBM path tk_fdk_device
    on the same projections (same launches in the same order);
  * several chunks differ from it only by FP32 accumulation order (each
    chunk's sum is added to the volume): relative RMSE <= 2e-6, for chunk
    sizes that divide N and that do not;
  * raw uint16 counts against the FP64 oracle of the raw counts (the
    streamed oracle): FP32 storage <= 1e-4, FP16 storage <= 5e-4;
  * pageable host memory gives the same volume as page-locked memory.
"""
import numpy as np
import pytest

from _util import rel_rmse, small_geometry
from tomokvas_gb300 import _lib, device
from tomokvas_gb300.phantom import counts_u16, head_phantom

pytestmark = pytest.mark.gpu

I0 = 60000.0


@pytest.fixture(scope="module")
def case(orc, cuda):
    """Head phantom, 100 x 64 x 72 projections (projection-major), 56 x 60 x 48 volume."""
    g = small_geometry(W=64, N=100, H=72, vol=(56, 60, 48))
    G = orc.geom_from(g)
    ell = head_phantom(g.fov_radius_cm * 0.85, seed=11)
    proj = orc.project_ellipsoids(ell, G, "proj")  # [N][H][W]
    return g, G, proj


def pinned(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory()


@pytest.mark.parametrize("chunk", [7, 25, 100, 512])
def test_stream_matches_in_hbm_path(case, chunk):
    import torch

    g, G, proj = case
    ref = device.fdk_device(g, torch.from_numpy(proj).cuda(), _lib.TK_INPUT_F32, _lib.TK_LAYOUT_PROJECTION,
                            precision=_lib.TK_F32)
    got = device.fdk_stream(g, pinned(proj, torch), _lib.TK_INPUT_F32, precision=_lib.TK_F32, chunk=chunk)
    torch.cuda.synchronize()
    a, b = got.cpu().numpy(), ref.cpu().numpy()
    if chunk >= g.N:
        np.testing.assert_array_equal(a, b)
    else:
        assert rel_rmse(a, b) < 2e-6
    assert device.device_error_flags() == 0


@pytest.mark.parametrize("precision,tol", [(_lib.TK_F32, 1e-4), (_lib.TK_F16, 5e-4)])
def test_stream_u16_vs_fp64(orc, case, precision, tol):
    import torch

    g, G, proj = case
    raw = counts_u16(proj, I0, seed=12)  # [N][H][W] uint16
    ff = device.flatfield(flat_value=I0, A=1.0, B=0.0, invert=True, floor_counts=0.5)
    h = pinned(raw.view(np.int16), torch)
    vol = device.fdk_stream(g, h, _lib.TK_INPUT_U16, ff=ff, window=_lib.TK_WINDOW_HANN, precision=precision,
                            chunk=32)
    torch.cuda.synchronize()
    ref = orc.fdk_u16_f64_sampled(raw, G, I0, window="hann", zlist=np.arange(g.Z, dtype=np.int32))
    assert rel_rmse(vol.cpu().numpy(), ref) < tol
    assert device.device_error_flags() == 0


def test_stream_pageable_equals_pinned(case):
    import torch

    g, G, proj = case
    a = device.fdk_stream(g, pinned(proj, torch), _lib.TK_INPUT_F32, precision=_lib.TK_F16, chunk=30)
    b = device.fdk_stream(g, np.ascontiguousarray(proj), _lib.TK_INPUT_F32, precision=_lib.TK_F16, chunk=30)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())


@pytest.mark.parametrize("chunk", [8, 44, 200])
def test_stream_quarter_turn_chunks(orc, cuda, chunk):
    """FP16 storage on a square centred volume with N = 120: each chunk is the
    four ranges of chunk/4 projections a quarter turn apart (2, 11 with a
    ragged last chunk of 8, or all 30), backprojected by the quarter-turn
    kernel from the chunk's compact image.  Raw counts with a scalar flat
    field (a storage scale known before the data) make every chunk's FP16
    entries those of the whole image: one chunk is bit-identical to the in-HBM
    path, more chunks differ by FP32 accumulation order only.  The general
    FP32-interpolation walk gives other bits (another kernel ran)."""
    import torch

    g = small_geometry(W=64, N=120, H=64, vol=(64, 64, 40))
    G = orc.geom_from(g)
    proj = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=13), G, "proj")
    raw = counts_u16(proj, I0, seed=14)
    ff = device.flatfield(flat_value=I0, A=1.0, B=0.0, invert=True, floor_counts=0.5)
    d_raw = torch.from_numpy(raw.view(np.int16)).cuda()
    ref = device.fdk_device(g, d_raw, _lib.TK_INPUT_U16, _lib.TK_LAYOUT_PROJECTION, ff=ff,
                            window=_lib.TK_WINDOW_HANN, precision=_lib.TK_F16).cpu().numpy()
    got = device.fdk_stream(g, pinned(raw.view(np.int16), torch), _lib.TK_INPUT_U16, ff=ff,
                            window=_lib.TK_WINDOW_HANN, precision=_lib.TK_F16, chunk=chunk).cpu().numpy()
    L = _lib.load()
    names = [L.tk_bp_variant_name(i).decode() for i in range(L.tk_bp_variant_count())]
    gen = next(i for i, n in enumerate(names) if n.startswith("cimg_f32i<f16,"))
    try:
        _lib.check(L.tk_bp_select_variant(gen))
        general = device.fdk_stream(g, pinned(raw.view(np.int16), torch), _lib.TK_INPUT_U16, ff=ff,
                                    window=_lib.TK_WINDOW_HANN, precision=_lib.TK_F16,
                                    chunk=chunk).cpu().numpy()
    finally:
        _lib.check(L.tk_bp_select_variant(-1))
    if chunk >= g.N:
        np.testing.assert_array_equal(got, ref)
    else:
        assert rel_rmse(got, ref) < 2e-6
    assert not np.array_equal(got, general)
    assert rel_rmse(got, general) < 1e-5
    assert device.device_error_flags() == 0
