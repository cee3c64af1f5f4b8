"""The ramp filter as a Toeplitz product on the tcgen05 tensor cores
(TK_FILTER_TOEPLITZ) against the shared-memory FFT form and the FP32
restatement of the reference's filter (fConvolution, FBPG/kernel.cu:557-781).

The product uses split-BF16 compensated operands (hi + lo parts of the data
and of the kernel, three products, FP32 accumulation in tensor memory), so it
differs from the FFT form by FP32-level rounding plus the dropped lo x lo
term (below 2^-16 relative per product).  Bounds, relative RMSE:
  filtered FP32 samples vs FFT form and vs the FP32 restatement   1e-4
  FP32 coefficient image vs FFT form: the sample values Q           1e-4,
    every entry value's error relative to the RMS sample value      1e-4
    (differences of samples carry the samples' absolute error)
  16-bit coefficient images: entries within 4 units of the format's
    rounding of the RMS value (the formats round the same values)
  whole FDK vs FP64 oracle: FP16 storage (the automatic choice)     5e-4;
    FP32 storage with the product forced                            5e-5
The automatic selection takes the product for 16-bit storage only: its
accuracy (about 2e-5 on filtered values) is below 16-bit rounding but above
the FP32 forms' 1e-5 reconstruction bound, which keep the FFT.
"""
import numpy as np
import pytest

from _util import rel_rmse, small_geometry
from tomokvas_gb300 import _lib, device
from tomokvas_gb300.phantom import counts_u16, head_phantom

pytestmark = pytest.mark.gpu

TOEP_RMSE = 1e-4


def to_dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def with_form(form, fn):
    L = _lib.load()
    _lib.check(L.tk_filter_select_form(form))
    try:
        return fn()
    finally:
        _lib.check(L.tk_filter_select_form(_lib.TK_FILTER_AUTO))


def test_form_selection():
    """W <= 512 can take the tensor-core form; wider rows always take the FFT."""
    L = _lib.load()
    try:
        _lib.check(L.tk_filter_select_form(_lib.TK_FILTER_TOEPLITZ))
        assert L.tk_filter_form_for(256, _lib.TK_F16) == _lib.TK_FILTER_TOEPLITZ
        assert L.tk_filter_form_for(1024, _lib.TK_F16) == _lib.TK_FILTER_FFT
        _lib.check(L.tk_filter_select_form(_lib.TK_FILTER_FFT))
        assert L.tk_filter_form_for(256, _lib.TK_F16) == _lib.TK_FILTER_FFT
    finally:
        _lib.check(L.tk_filter_select_form(_lib.TK_FILTER_AUTO))
    assert L.tk_filter_select_form(7) == _lib.TK_ERR_INVALID


# widths covering one to four 128-column output tiles, ragged widths and K extents
@pytest.mark.parametrize("W", [8, 24, 64, 130, 200, 256, 300, 384, 500, 512])
@pytest.mark.parametrize("window", ["ramlak", "hann"])
def test_toeplitz_filter_matches_fft(orc, cuda, W, window):
    """FP32 samples: N x H = 24 x 70 rows (row tiles spanning projections),
    sinogram-major random input."""
    import torch

    g = small_geometry(W=W, N=24, H=70, vol=(16, 16, 8))
    G = orc.geom_from(g)
    rng = np.random.default_rng(W)
    sino = rng.normal(size=(g.H, g.N, g.W)).astype(np.float32)
    d = to_dev(sino, torch)
    wn = _lib.WINDOWS[window]

    def run():
        q, _ = device.filter_projections(g, d, window=wn)
        torch.cuda.synchronize()
        return q.cpu().numpy()[:, :, :g.W]

    qt = with_form(_lib.TK_FILTER_TOEPLITZ, run)
    qf = with_form(_lib.TK_FILTER_FFT, run)
    q_ref = np.transpose(orc.filter_f32(orc.weight_f32(sino, G), G, window), (1, 0, 2))
    assert device.device_error_flags() == 0
    assert not np.array_equal(qt, qf)  # the tensor-core form ran
    assert rel_rmse(qt, qf) < TOEP_RMSE
    assert rel_rmse(qt, q_ref) < TOEP_RMSE


@pytest.mark.parametrize("W,N", [(200, 300), (384, 200)])
def test_toeplitz_many_tiles_per_cta(cuda, W, N):
    """FP32 samples from N x 256 detector rows: hundreds of row tiles, four to
    six per CTA, so both tensor-memory accumulators are reused (a tile's MMAs
    wait for the epilogue of the tile two before) and both epilogue sets take
    chunks of several tiles."""
    import torch

    g = small_geometry(W=W, N=N, H=256, vol=(16, 16, 8))
    rng = np.random.default_rng(W + N)
    sino = rng.normal(size=(g.H, g.N, g.W)).astype(np.float32)
    d = to_dev(sino, torch)

    def run():
        q, _ = device.filter_projections(g, d, window=_lib.TK_WINDOW_HANN)
        torch.cuda.synchronize()
        return q.cpu().numpy()[:, :, :g.W]

    qt = with_form(_lib.TK_FILTER_TOEPLITZ, run)
    qf = with_form(_lib.TK_FILTER_FFT, run)
    assert device.device_error_flags() == 0
    assert not np.array_equal(qt, qf)
    assert rel_rmse(qt, qf) < TOEP_RMSE
    # every row, not only on average: the worst detector row stays within the bound
    per_row = np.sqrt(np.mean((qt - qf) ** 2, axis=2) / np.maximum(np.mean(qf ** 2, axis=2), 1e-30))
    assert float(per_row.max()) < 10 * TOEP_RMSE


def test_toeplitz_many_tiles_u16_f16(cuda):
    """Raw uint16 frames into FP16 coefficients at W = 512 (64-row tiles, four
    or five per CTA): the uint16 producers and the coefficient epilogue over
    reused accumulators, against the FFT form."""
    import torch

    g = small_geometry(W=512, N=160, H=256, vol=(16, 16, 8))
    rng = np.random.default_rng(5)
    raw = rng.integers(2000, 60000, size=(g.N, g.H, g.W)).astype(np.uint16)
    d = torch.from_numpy(raw.view(np.int16)).cuda()
    ff = device.flatfield(flat_value=60000.0)

    def run():
        q, s = device.filter_projections(g, d, _lib.TK_INPUT_U16, _lib.TK_LAYOUT_PROJECTION, ff=ff,
                                         window=_lib.TK_WINDOW_HANN, precision=_lib.TK_F16)
        torch.cuda.synchronize()
        return q.cpu().numpy(), float(s.item())

    (qt, st), (qf, sf) = with_form(_lib.TK_FILTER_TOEPLITZ, run), with_form(_lib.TK_FILTER_FFT, run)
    assert st == sf
    et, ef = decode_entries(qt, _lib.TK_F16, g), decode_entries(qf, _lib.TK_F16, g)
    assert device.device_error_flags() == 0
    assert not np.array_equal(et, ef)
    rms = np.sqrt(np.mean(ef ** 2))
    assert np.sqrt(np.mean((et - ef) ** 2)) < 4 * 2.0 ** -10 * rms


def decode_entries(raw, precision, g):
    """Coefficient image bytes [N][H][pitch] -> float64 (Q, dU, dV, dUV) of columns < W."""
    W = g.W
    if precision == _lib.TK_F32_COEF:
        e = raw.view(np.float32).reshape(g.N, g.H, -1, 4)
        return e[:, :, :W, :].astype(np.float64)
    dt = np.float16 if precision == _lib.TK_F16 else None
    u = raw.view(np.uint16).reshape(g.N, g.H, -1, 4)[:, :, :W, :]
    if dt is not None:
        v = u.view(np.float16).astype(np.float64)
    else:
        v = (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    # {(Q, dV), (dU, dUV)} -> (Q, dU, dV, dUV)
    return v[..., [0, 2, 1, 3]]


@pytest.mark.parametrize("precision", ["f32c", "f16", "bf16"])
@pytest.mark.parametrize("W,layout", [(130, "projection"), (384, "sinogram"), (512, "projection")])
def test_toeplitz_coefficient_images(orc, cuda, precision, W, layout):
    """Coefficient images (the entry's next row and next column come from the
    staged accumulator: tile, warp and projection boundaries) from raw
    uint16 counts, against the FFT form's image."""
    import torch

    g = small_geometry(W=W, N=12, H=50, vol=(16, 16, 8))
    G = orc.geom_from(g)
    proj = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=W), G, "proj")
    raw = counts_u16(proj, 60000.0, seed=W + 1)
    if layout == "sinogram":
        raw = np.ascontiguousarray(np.transpose(raw, (1, 0, 2)))
    d = torch.from_numpy(raw.view(np.int16)).cuda()
    ff = device.flatfield(flat_value=60000.0)
    prec = _lib.PRECISIONS[precision]

    def run():
        q, s = device.filter_projections(g, d, _lib.TK_INPUT_U16, _lib.LAYOUTS[layout], ff=ff,
                                         window=_lib.TK_WINDOW_HANN, precision=prec)
        torch.cuda.synchronize()
        return q.cpu().numpy(), float(s.item())

    (qt, st), (qf, sf) = with_form(_lib.TK_FILTER_TOEPLITZ, run), with_form(_lib.TK_FILTER_FFT, run)
    assert st == sf
    et, ef = decode_entries(qt, prec, g), decode_entries(qf, prec, g)
    assert device.device_error_flags() == 0
    assert not np.array_equal(et, ef)
    if prec == _lib.TK_F32_COEF:
        assert rel_rmse(et[..., 0], ef[..., 0]) < TOEP_RMSE
        assert np.sqrt(np.mean((et - ef) ** 2)) < TOEP_RMSE * np.sqrt(np.mean(ef[..., 0] ** 2))
    else:
        ulp = 2.0 ** (-10 if prec == _lib.TK_F16 else -7)
        rms = np.sqrt(np.mean(ef ** 2))
        assert np.sqrt(np.mean((et - ef) ** 2)) < 4 * ulp * rms


def test_toeplitz_fdk_vs_fp64(orc, cuda):
    """Whole FDK through tk_fdk_device: with FP16 storage the automatic
    selection takes the tensor-core filter (W = 64) and meets the FP16 bound;
    with FP32 storage it keeps the FFT, and the product forced stays within
    5e-5 of FP64."""
    import torch

    g = small_geometry(W=64, N=120, H=64, vol=(64, 64, 48))
    G = orc.geom_from(g)
    sino = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=3), G, "sino")
    d = to_dev(sino, torch)
    L = _lib.load()
    assert L.tk_filter_form_for(g.W, _lib.TK_F16) == _lib.TK_FILTER_TOEPLITZ
    assert L.tk_filter_form_for(g.W, _lib.TK_BF16) == _lib.TK_FILTER_TOEPLITZ
    assert L.tk_filter_form_for(g.W, _lib.TK_F32) == _lib.TK_FILTER_FFT
    assert L.tk_filter_form_for(g.W, _lib.TK_F32_COEF) == _lib.TK_FILTER_FFT

    def run(prec):
        def f():
            v = device.fdk_device(g, d, precision=prec)
            torch.cuda.synchronize()
            return v.cpu().numpy()
        return f

    ref = orc.fdk_f64(sino, G)
    v16 = run(_lib.TK_F16)()
    v16f = with_form(_lib.TK_FILTER_FFT, run(_lib.TK_F16))
    vt = with_form(_lib.TK_FILTER_TOEPLITZ, run(_lib.TK_F32))
    vf = with_form(_lib.TK_FILTER_FFT, run(_lib.TK_F32))
    assert device.device_error_flags() == 0
    assert not np.array_equal(v16, v16f)
    assert rel_rmse(v16, ref) < 5e-4
    assert rel_rmse(vt, ref) < 5e-5 and rel_rmse(vt, vf) < 5e-5
    assert rel_rmse(vf, ref) < 1e-5
