"""GPU parity: every stage of the CUDA path against the CPU oracle.

All device work goes through libtk_fdk.so's C ABI; torch only allocates
device memory.  Tolerances (relative RMSE over the volume, max-abs relative
to max |volume|):
  noise-free analytic projections:
    FP32 path vs FP32 restatement of the reference   rmse <= 1e-5, max <= 1e-4
    FP32 path vs FP64 oracle                          rmse <= 1e-5
  raw Poisson counts (noisy): FP32 interpolation-weight rounding of the
  reference algorithm itself dominates (its FP32 restatement sits ~3e-5 from
  FP64 on the small phantom), so
    FP32 path vs FP64 oracle   rmse <= max(1e-5, 2 x restatement-vs-FP64) and <= 1e-4
  16-bit storage (FP32 math) vs FP64 oracle:
    FP16 rmse <= 5e-4, BF16 rmse <= 4e-3
"""
import numpy as np
import pytest

from _util import max_abs, rel_rmse, small_geometry
from tomokvas_gb300 import _lib, device
from tomokvas_gb300.fbp import FilteredBackProjection, VolumeSink
from tomokvas_gb300.phantom import counts_u16, head_phantom, random_ellipsoids

pytestmark = pytest.mark.gpu

F32_RMSE, F32_MAX, F16_RMSE, BF16_RMSE = 1e-5, 1e-4, 5e-4, 4e-3
TARGET_RMSE = 1e-4  # FP32 form vs FP64 oracle, any input


def noisy_tol(rest_err):
    """FP32 bound on noisy input: no worse than twice the reference algorithm's own FP32 error."""
    return min(TARGET_RMSE, max(F32_RMSE, 2.0 * rest_err))


def exact_centring(orc, g):
    zoff = orc.zblocks(orc.geom_from(g))
    if len(zoff) * g.zb < g.Z:
        return False
    z = np.arange(g.Z)
    return bool(np.all(np.float32(z % g.zb) + zoff[z // g.zb] == np.float32(z - (g.Z - 1) / 2.0)))


def to_dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def case(orc, cuda):
    """Small head phantom, 120 x 64^2 projections, 64^3 volume (exact Z centring)."""
    g = small_geometry()
    G = orc.geom_from(g)
    ell = head_phantom(g.fov_radius_cm * 0.9, seed=1)
    sino = orc.project_ellipsoids(ell, G, "sino")  # [H][N][W], FP64 analytic
    return g, G, ell, sino


def test_phantom_projector_matches_oracle(orc, cuda, case):
    import torch

    g, G, ell, sino = case
    d = device.phantom_project(g, ell, _lib.TK_LAYOUT_SINOGRAM)
    torch.cuda.synchronize()
    assert rel_rmse(d.cpu().numpy(), sino) < 1e-5


@pytest.mark.parametrize("window", ["ramlak", "shepp_logan", "hann"])
@pytest.mark.parametrize("layout", ["sinogram", "projection"])
def test_filter_stage_matches_oracle(orc, cuda, case, window, layout):
    import torch

    g, G, ell, sino = case
    q_ref = orc.filter_f32(orc.weight_f32(sino, G), G, window)  # [H][N][W], reference scale
    src = sino if layout == "sinogram" else np.transpose(sino, (1, 0, 2))
    q, s = device.filter_projections(g, to_dev(src, torch), _lib.TK_INPUT_F32, _lib.LAYOUTS[layout],
                                     window=_lib.WINDOWS[window])
    torch.cuda.synchronize()
    qd = q.cpu().numpy()[:, :, :g.W]
    assert float(s.item()) == 1.0
    assert rel_rmse(qd, np.transpose(q_ref, (1, 0, 2))) < 2e-6


@pytest.mark.parametrize("W", [24, 33, 130, 300, 768, 1500, 2048, 4096])
def test_filter_every_pad_length(orc, cuda, W):
    """Every FFT pass schedule of the filter: p = 64 (16,4) ... 8192 (16,16,16,2)."""
    import torch

    g = small_geometry(W=W, N=3, H=5, vol=(16, 16, 8))
    G = orc.geom_from(g)
    rng = np.random.default_rng(W)
    sino = rng.normal(size=(g.H, g.N, g.W)).astype(np.float32)
    q_ref = orc.filter_f32(orc.weight_f32(sino, G), G, "hann")
    q, _ = device.filter_projections(g, to_dev(sino, torch), window=_lib.TK_WINDOW_HANN)
    torch.cuda.synchronize()
    assert rel_rmse(q.cpu().numpy()[:, :, :g.W], np.transpose(q_ref, (1, 0, 2))) < 2e-6


def coefficients_from_samples(q):
    """(Q, dU, dV, dUV) of every cell of q[N][H][W], samples outside are 0."""
    qp = np.zeros((q.shape[0], q.shape[1] + 1, q.shape[2] + 1), dtype=np.float64)
    qp[:, :-1, :-1] = q
    Q = qp[:, :-1, :-1]
    dU = qp[:, :-1, 1:] - Q
    dV = qp[:, 1:, :-1] - Q
    dUV = qp[:, 1:, 1:] - qp[:, 1:, :-1] - dU
    return np.stack([Q, dU, dV, dUV], axis=-1)


@pytest.mark.parametrize("precision", ["f32c", "f16", "bf16"])
@pytest.mark.parametrize("H", [64, 130])  # 130: a work unit boundary inside the detector and a short last unit
def test_filter_writes_coefficient_image(orc, cuda, precision, H):
    import torch

    g = small_geometry(W=60, N=7, H=H, vol=(32, 32, 32))
    G = orc.geom_from(g)
    rng = np.random.default_rng(9)
    sino = rng.normal(size=(g.H, g.N, g.W)).astype(np.float32)
    q_ref = np.transpose(orc.filter_f32(orc.weight_f32(sino, G), G), (1, 0, 2)).astype(np.float64)
    exp = coefficients_from_samples(q_ref)  # [N][H][W][4]
    prec = _lib.PRECISIONS[precision]
    q, s = device.filter_projections(g, to_dev(sino, torch), precision=prec)
    torch.cuda.synchronize()
    raw = q.cpu().numpy().view(np.uint8)
    if prec == _lib.TK_F32_COEF:
        got = raw.view(np.float32).reshape(g.N, g.H, g.W, 4).astype(np.float64)
        tol = 2e-6
    else:
        Wc = (g.W + 1) & ~1
        h = raw.view(np.uint16).reshape(g.N, g.H, Wc, 4)[:, :, :g.W]
        if prec == _lib.TK_F16:
            vals = h.view(np.float16).astype(np.float64)
        else:
            vals = (h.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
        got = vals[..., [0, 2, 1, 3]] / float(s.item())  # stored as (Q, dV), (dU, dUV)
        tol = 2e-3 if prec == _lib.TK_F16 else 1.5e-2
    for k in range(4):
        scale = np.sqrt(np.mean(exp[..., 0] ** 2))
        assert np.sqrt(np.mean((got[..., k] - exp[..., k]) ** 2)) < tol * scale, (precision, k)


def test_bp_stage_matches_oracle(orc, cuda, case):
    import torch

    g, G, ell, sino = case
    q_ref = orc.filter_f32(orc.weight_f32(sino, G), G)
    vol_ref = orc.bp_f32(q_ref, G)
    qp = np.zeros((g.N, g.H, device.row_pitch(g.W)), dtype=np.float32)
    qp[:, :, :g.W] = np.transpose(q_ref, (1, 0, 2))
    vol = device.backproject(g, to_dev(qp, torch), None)
    torch.cuda.synchronize()
    v = vol.cpu().numpy()
    assert rel_rmse(v, vol_ref) < 2e-6
    assert max_abs(v, vol_ref) < 2e-5 * np.abs(vol_ref).max()
    assert device.device_error_flags() == 0


def test_every_bp_variant_matches_oracle(orc, cuda, case):
    """All compiled backprojection variants (tile shape / pipeline) agree with the oracle."""
    import torch

    from tomokvas_gb300._lib import check, load

    g, G, ell, sino = case
    L = load()
    v64 = orc.fdk_f64(sino, G)
    v32 = orc.fdk_f32(sino, G)
    d_in = to_dev(sino, torch)
    try:
        for i in range(L.tk_bp_variant_count()):
            prec = L.tk_bp_variant_precision(i)
            check(L.tk_bp_select_variant(i))
            v = device.fdk_device(g, d_in, precision=prec)
            torch.cuda.synchronize()
            v = v.cpu().numpy()
            name = L.tk_bp_variant_name(i).decode()
            if prec in (_lib.TK_F32, _lib.TK_F32_COEF):
                assert rel_rmse(v, v32) < F32_RMSE, name
            else:
                assert rel_rmse(v, v64) < (F16_RMSE if prec == _lib.TK_F16 else BF16_RMSE), name
            assert device.device_error_flags() == 0, name
    finally:
        check(L.tk_bp_select_variant(-1))


def _names(L):
    return [L.tk_bp_variant_name(i).decode() for i in range(L.tk_bp_variant_count())]


def _general(names, pn):
    """Index of the general (non-quarter-turn) default walk of a storage format."""
    if pn == "f32c":
        return next(i for i, n in enumerate(names) if n.startswith("cimg_x2<f32c"))
    return next(i for i, n in enumerate(names) if n.startswith(f"cimg_f32i<{pn},"))


@pytest.mark.parametrize("Z", [40, 10])  # a moved-down last z chunk; a chunk shorter than 16 slices
@pytest.mark.parametrize("pn,prec,tol", [("f16", _lib.TK_F16, F16_RMSE), ("bf16", _lib.TK_BF16, BF16_RMSE),
                                         ("f32c", _lib.TK_F32_COEF, F32_RMSE)])
def test_quarter_turn_kernel(orc, cuda, Z, pn, prec, tol):
    """A square, centred, unflipped volume with N divisible by 4 runs the
    quarter-turn kernel of the storage format (one geometry for four tiles and
    four projections, FP32 interpolation; for FP32 coefficients, where it is
    slower than the general walk, when selected); it meets the format's bound against
    FP64 and stays within rounding of the general FP32-interpolation walk.  An
    x flip breaks the symmetry: the general walk runs, bit for bit.  Every
    FP32-interpolation quarter-turn variant of the format with the same slices
    per tile (tile height, stage count, box capacity) gives the same bits; the
    8-slice tiles agree to FP32 rounding."""
    import torch

    L = _lib.load()
    names = _names(L)
    gen = _general(names, pn)
    quads = [i for i, n in enumerate(names) if n.startswith(f"quad<{pn},") and ",f32i," in n]
    assert quads
    for flip in (0, 1):
        g = small_geometry(W=64, N=120, H=64, vol=(64, 64, Z), dirx=flip)
        G = orc.geom_from(g)
        sino = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=11), G, "sino")
        d_in = to_dev(sino, torch)
        vols = []
        # FP32 coefficients run the general walk by default (faster); their quarter-turn form is selected
        first = quads[0] if prec == _lib.TK_F32_COEF else -1
        try:
            for sel in [first, gen] + quads:
                _lib.check(L.tk_bp_select_variant(sel))
                vols.append(device.fdk_device(g, d_in, precision=prec).cpu().numpy())
        finally:
            _lib.check(L.tk_bp_select_variant(-1))
        assert device.device_error_flags() == 0
        tz = [int(names[i].split(",")[3]) for i in quads]  # slices per tile: a pair's row coordinate
        for v, t in zip(vols[2:], tz):                      # is formed from the tile's first slice
            if t == tz[0] or flip:
                np.testing.assert_array_equal(v, vols[0])
            else:
                assert rel_rmse(v, vols[0]) < 1e-6
        if flip:
            np.testing.assert_array_equal(vols[0], vols[1])
        else:
            assert not np.array_equal(vols[0], vols[1])  # a different kernel ran
            ref = orc.fdk_f64(sino, G) if prec != _lib.TK_F32_COEF else orc.fdk_f32(sino, G)
            assert rel_rmse(vols[0], ref) < tol
            # the same arithmetic on the same stored values, geometry of the turned columns taken
            # from the base column (angles a quarter turn apart agree to 1e-5 rad)
            assert rel_rmse(vols[0], vols[1]) < 2e-6


@pytest.mark.parametrize("Z", [40, 10])
def test_quarter_turn_half_math_forms(orc, cuda, Z):
    """The selectable FP16 half-math forms (FP16 interpolation arithmetic):
    every quarter-turn half-math variant (row interpolation by HFMA2 on
    regrouped halves or by FP16 FMAs on half-selected operands) gives the same
    bits, and so do the two general half-math walks (cimg_h2, cimg_h3); both
    meet the FP16 bound.  The default FP32-interpolation form is at least as
    close to FP64 on this case."""
    import torch

    L = _lib.load()
    names = _names(L)
    h2 = next(i for i, n in enumerate(names) if n.startswith("cimg_h2<f16"))
    h3 = next(i for i, n in enumerate(names) if n.startswith("cimg_h3<f16"))
    hq = [i for i, n in enumerate(names) if n.startswith("quad<f16,") and ",h16row" in n]
    assert len(hq) >= 2
    g = small_geometry(W=64, N=120, H=64, vol=(64, 64, Z))
    G = orc.geom_from(g)
    sino = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=11), G, "sino")
    d_in = to_dev(sino, torch)
    vols = []
    try:
        for sel in [-1, h2, h3] + hq:
            _lib.check(L.tk_bp_select_variant(sel))
            vols.append(device.fdk_device(g, d_in, precision=_lib.TK_F16).cpu().numpy())
    finally:
        _lib.check(L.tk_bp_select_variant(-1))
    assert device.device_error_flags() == 0
    np.testing.assert_array_equal(vols[2], vols[1])
    for v in vols[4:]:
        np.testing.assert_array_equal(v, vols[3])
    ref = orc.fdk_f64(sino, G)
    assert rel_rmse(vols[3], ref) < F16_RMSE and rel_rmse(vols[1], ref) < F16_RMSE
    assert rel_rmse(vols[3], vols[1]) < 2e-4
    assert rel_rmse(vols[0], ref) <= rel_rmse(vols[3], ref) * 1.05


@pytest.mark.parametrize("N,rot,Z", [(8, 0.3, 24),       # two projections per quarter, rotated scan
                                      (360, 1.0, 40),     # a rotation of about a radian
                                      (3200, 0.0, 8)])    # the most angles one launch carries
def test_quarter_turn_kernel_angle_sets(orc, cuda, N, rot, Z):
    """The quarter-turn kernel on small and large angle sets and with a
    rotation offset (the angles stay in quarter-turn sets): it runs (other
    bits than the general FP32-interpolation walk) and meets the FP16 bound
    against FP64."""
    import torch

    L = _lib.load()
    gen = _general(_names(L), "f16")
    g = small_geometry(W=64, N=N, H=64, vol=(64, 64, Z), rot=rot)
    G = orc.geom_from(g)
    sino = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=21), G, "sino")
    d_in = to_dev(sino, torch)
    vols = []
    try:
        for sel in (-1, gen):
            _lib.check(L.tk_bp_select_variant(sel))
            vols.append(device.fdk_device(g, d_in, precision=_lib.TK_F16).cpu().numpy())
    finally:
        _lib.check(L.tk_bp_select_variant(-1))
    assert device.device_error_flags() == 0
    assert not np.array_equal(vols[0], vols[1])
    assert rel_rmse(vols[0], orc.fdk_f64(sino, G)) < F16_RMSE
    assert rel_rmse(vols[0], vols[1]) < 1e-5


def test_quarter_turn_wide_boxes(orc, cuda):
    """At scale 1.5 a 16x16x16 tile's footprint (46 x 32 entries, 11.8 KB)
    exceeds the 6 KB slots of the default FP16 quarter-turn kernel (16x8
    tiles) and the 8 KB slots of its 16x16 form: with no variant selected the
    two-stage 13.5 KB form runs (the same bits as selecting it), while
    selecting the 8 KB form falls back to the general FP32-interpolation
    walk."""
    import torch

    L = _lib.load()
    names = _names(L)
    gen = _general(names, "f16")
    narrow = next(i for i, n in enumerate(names) if n.startswith("quad<f16,") and "cap8192" in n and ",f32i," in n)
    wide = next(i for i, n in enumerate(names) if n.startswith("quad<f16,") and "cap13824" in n and ",f32i," in n)
    g = small_geometry(W=96, N=120, H=96, vol=(64, 64, 40), voxel_mm=1.2)
    G = orc.geom_from(g)
    sino = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=23), G, "sino")
    d_in = to_dev(sino, torch)
    vols = {}
    try:
        for sel in (-1, wide, narrow, gen):
            _lib.check(L.tk_bp_select_variant(sel))
            vols[sel] = device.fdk_device(g, d_in, precision=_lib.TK_F16).cpu().numpy()
    finally:
        _lib.check(L.tk_bp_select_variant(-1))
    assert device.device_error_flags() == 0
    np.testing.assert_array_equal(vols[-1], vols[wide])
    np.testing.assert_array_equal(vols[narrow], vols[gen])
    assert not np.array_equal(vols[-1], vols[gen])
    assert rel_rmse(vols[-1], orc.fdk_f64(sino, G)) < F16_RMSE


def test_packed_variants_equal_scalar(orc, cuda, case):
    """The *_x2 variants walk two slices per step with packed FP32 but do the
    same IEEE operations per voxel as the scalar walk: identical bits."""
    import torch

    g, G, ell, sino = case
    g = g.replace(Z=100)  # full chunks and a moved-down last chunk
    L = _lib.load()
    names = {i: L.tk_bp_variant_name(i).decode() for i in range(L.tk_bp_variant_count())}
    pairs = [(i, j) for i, n in names.items() if "_x2<" in n
             for j, m in names.items() if m == n.replace("_x2<", "<")]
    assert pairs
    try:
        for i, j in pairs:
            prec = L.tk_bp_variant_precision(i)
            q, sc = device.filter_projections(g, to_dev(sino, torch), precision=prec)
            sc = sc if prec in (_lib.TK_F16, _lib.TK_BF16) else None
            out = []
            for vi in (i, j):
                _lib.check(L.tk_bp_select_variant(vi))
                out.append(device.backproject(g, q, sc, prec).cpu().numpy())
            np.testing.assert_array_equal(out[0], out[1])
    finally:
        _lib.check(L.tk_bp_select_variant(-1))
    assert device.device_error_flags() == 0


def test_fdk_f32_matches_restatement_and_fp64(orc, cuda, case):
    import torch

    g, G, ell, sino = case
    vol = device.fdk_device(g, to_dev(sino, torch))
    torch.cuda.synchronize()
    v = vol.cpu().numpy()
    v32 = orc.fdk_f32(sino, G)
    v64 = orc.fdk_f64(sino, G)
    assert rel_rmse(v, v32) < F32_RMSE and max_abs(v, v32) < F32_MAX * np.abs(v32).max()
    assert rel_rmse(v, v64) < F32_RMSE


@pytest.mark.parametrize("precision,tol", [("f16", F16_RMSE), ("bf16", BF16_RMSE), ("f32c", F32_RMSE)])
def test_fdk_storage_formats_vs_fp64(orc, cuda, case, precision, tol):
    import torch

    g, G, ell, sino = case
    vol = device.fdk_device(g, to_dev(sino, torch), precision=_lib.PRECISIONS[precision])
    torch.cuda.synchronize()
    v64 = orc.fdk_f64(sino, G)
    assert rel_rmse(vol.cpu().numpy(), v64) < tol
    assert device.device_error_flags() == 0


@pytest.mark.parametrize("kw", [
    dict(W=60, N=50, H=45, vol=(50, 37, 29)),                  # ragged sizes, W not a multiple of 8
    dict(W=64, N=90, H=64, vol=(48, 48, 48), voxel_mm=1.2),   # scale 1.5
    dict(W=64, N=72, H=70, vol=(40, 40, 40), dirx=1, diry=1, dirz=1, rot=0.3),
    dict(W=66, N=40, H=40, vol=(32, 32, 32)),                 # W = 2 mod 4 (|FFT| filter)
])
def test_fdk_geometries(orc, cuda, kw):
    import torch

    g = small_geometry(**kw)
    G = orc.geom_from(g)
    ell = head_phantom(g.fov_radius_cm * 0.8, seed=5)
    sino = orc.project_ellipsoids(ell, G, "sino")
    vol = device.fdk_device(g, to_dev(sino, torch))
    torch.cuda.synchronize()
    v = vol.cpu().numpy()
    assert device.device_error_flags() == 0
    v64 = orc.fdk_f64(sino, G)
    assert rel_rmse(v, v64) < F32_RMSE
    if exact_centring(orc, g):  # the restatement follows the reference's block schedule
        v32 = orc.fdk_f32(sino, G)
        assert rel_rmse(v, v32) < F32_RMSE


def test_u16_log_path(orc, cuda, case):
    import torch

    g, G, ell, sino = case
    raw = counts_u16(np.transpose(sino, (1, 0, 2)), 60000.0, seed=7)  # [N][H][W]
    ff = device.flatfield(flat_value=60000.0, A=1.0, B=0.0, invert=True, floor_counts=0.5)
    vol = device.fdk_device(g, to_dev(raw, torch), _lib.TK_INPUT_U16, _lib.TK_LAYOUT_PROJECTION, ff=ff,
                            window=_lib.TK_WINDOW_HANN)
    torch.cuda.synchronize()
    p = orc.log_u16(raw, np.float32(60000.0))
    v64 = orc.fdk_f64(p, G, "hann")
    rest = rel_rmse(orc.fdk_f32(p, G, "hann"), v64)
    assert rel_rmse(vol.cpu().numpy(), v64) < noisy_tol(rest)


def test_u16_per_pixel_flat_dark(orc, cuda, case):
    import torch

    g, G, ell, sino = case
    rng = np.random.default_rng(1)
    flat = rng.uniform(50000, 60000, size=(g.H, g.W)).astype(np.float32)
    dark = rng.uniform(50, 150, size=(g.H, g.W)).astype(np.float32)
    lam = flat[None] * np.exp(-np.transpose(sino, (1, 0, 2))) + dark[None]
    raw = np.clip(np.round(lam), 0, 65535).astype(np.uint16)
    flat_d, dark_d = to_dev(flat, torch), to_dev(dark, torch)
    ff = device.flatfield(flat=flat_d, dark=dark_d, A=2.0, B=0.1, invert=True)
    vol = device.fdk_device(g, to_dev(raw, torch), _lib.TK_INPUT_U16, _lib.TK_LAYOUT_PROJECTION, ff=ff)
    torch.cuda.synchronize()
    p = orc.log_u16(raw, flat, dark, A=2.0, B=0.1, invert=True)
    v64 = orc.fdk_f64(p, G)
    rest = rel_rmse(orc.fdk_f32(p, G), v64)
    assert rel_rmse(vol.cpu().numpy(), v64) < noisy_tol(rest)


@pytest.mark.parametrize("W,layout", [(63, "projection"), (127, "sinogram"), (64, "sinogram")])
def test_u16_filter_stage_any_width(orc, cuda, W, layout):
    """The u16 load of the filter: 16-byte runs of 8 counts where rows are
    16-byte aligned (W = 64), one count at a time otherwise (odd W), in both
    layouts; the filtered rows equal the FP32 restatement of log, weight and
    filter (rsq flat field with dark, beam-hardening line and invert)."""
    import torch

    g = small_geometry(W=W, N=10, H=12, vol=(16, 16, 8))
    G = orc.geom_from(g)
    rng = np.random.default_rng(W)
    raw = rng.integers(200, 60000, size=(g.N, g.H, g.W), dtype=np.uint16)  # [N][H][W]
    src = raw if layout == "projection" else np.ascontiguousarray(np.transpose(raw, (1, 0, 2)))
    ff = device.flatfield(flat_value=61000.0, dark_value=120.0, A=1.3, B=0.05, invert=True, floor_counts=0.5)
    q, _ = device.filter_projections(g, to_dev(src.view(np.int16), torch), _lib.TK_INPUT_U16,
                                     _lib.LAYOUTS[layout], ff=ff, window=_lib.TK_WINDOW_HANN)
    torch.cuda.synchronize()
    p = orc.log_u16(raw, np.float32(61000.0), np.float32(120.0), A=1.3, B=0.05, invert=True)  # [H][N][W]
    q_ref = orc.filter_f32(orc.weight_f32(p, G), G, "hann")
    assert rel_rmse(q.cpu().numpy()[:, :, :g.W], np.transpose(q_ref, (1, 0, 2))) < 2e-6


def test_handle_block_schedule_matches_restatement(orc, cuda):
    """FilteredBackProjection mirror with a bin_siz-like sink, Z=255 / ZB=30
    (inexact reference Z centring) and the last-slice quirk case Z=33 / ZB=16."""
    for vol_shape, zb in [((48, 48, 255), 30), ((40, 40, 33), 16)]:
        g = small_geometry(W=64, N=60, H=300 if vol_shape[2] > 100 else 64, vol=vol_shape, zb=zb)
        G = orc.geom_from(g)
        ell = head_phantom(g.fov_radius_cm * 0.8, seed=2)
        sino = orc.project_ellipsoids(ell, G, "sino")
        out = VolumeSink(g.X, g.Y, g.Z, zb)
        fbp = FilteredBackProjection(raise_on_error=True)
        fbp.SetGPUid(0)
        fbp.SetBlockSize(zb)
        fbp.SetSinogramProperties(sino, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau)
        fbp.SetReconstructionProperties(out, g.X, g.cx, g.Y, g.cy, g.Z, g.cz, g.rot)
        fbp.SetScaleXYZ(g.scale)
        assert fbp.Initialize() == 0
        assert fbp.CalculateReconstruction() == 0
        fbp.close()
        v32 = orc.fdk_f32(sino, G)
        assert rel_rmse(out.volume, v32) < F32_RMSE
        assert max_abs(out.volume, v32) < F32_MAX * np.abs(v32).max()
        nblk = len(orc.zblocks(G))
        assert [b for b, _ in out.blocks_requested] == list(range(nblk))
        if (g.Z - 1) % zb == 0:
            assert np.all(out.volume[-1] == 0)


def test_collecting_angle_blocks_sum_to_full(orc, cuda, case):
    """Angle sub-blocks accumulated through the sink (para_TC.cpp:117-155)."""
    g, G, ell, sino = case
    n1 = g.N // 2
    out = VolumeSink(g.X, g.Y, g.Z, g.zb)
    for k, (b0, b1) in enumerate([(0, n1), (n1, g.N)]):
        part = np.ascontiguousarray(sino[:, b0:b1])
        fbp = FilteredBackProjection(raise_on_error=True)
        fbp.SetBlockSize(g.zb)
        fbp.SetCollecting(k > 0)
        fbp.SetSinogramProperties(part, g.W, g.cX, b1 - b0, g.H, g.cZ, g.dfi, g.D, g.tau)
        fbp.SetReconstructionProperties(out, g.X, g.cx, g.Y, g.cy, g.Z, g.cz, float(np.float32(b0 * g.dfi)))
        fbp.Initialize()
        fbp.CalculateReconstruction()
        fbp.close()
    full = orc.fdk_f64(sino, G)
    assert rel_rmse(out.volume, full) < F32_RMSE


def test_reconstruct_to_device_and_precisions(orc, cuda, case):
    import torch

    g, G, ell, sino = case
    v64 = orc.fdk_f64(sino, G)
    for prec, tol in [("f32", F32_RMSE), ("f16", F16_RMSE), ("f32c", F32_RMSE)]:
        fbp = FilteredBackProjection(raise_on_error=True)
        fbp.SetSinogramProperties(sino, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau)
        fbp.SetReconstructionProperties(None, g.X, g.cx, g.Y, g.cy, g.Z, g.cz, g.rot)
        fbp.SetPrecision(prec)
        fbp.Initialize()
        vol = torch.empty((g.Z, g.Y, g.X), dtype=torch.float32, device="cuda")
        fbp.ReconstructToDevice(vol.data_ptr())
        t = fbp.Timings()
        fbp.close()
        assert rel_rmse(vol.cpu().numpy(), v64) < tol
        assert t["bp_ms"] > 0 and t["filter_ms"] > 0


@pytest.mark.parametrize("prec,raw,layout", [("f16", True, "projection"), ("f32", True, "projection"),
                                             ("f32c", False, "projection"), ("f16", True, "sinogram"),
                                             ("f32", False, "sinogram")])
def test_handle_chunked_upload_equals_device_path(orc, cuda, prec, raw, layout):
    """Input with a storage scale known up front is uploaded in chunks that are
    filtered as they land (N = 150: chunks of 64, 64, 22; a sinogram-major
    chunk is packed into an [H][nb][W] block by a strided copy); the volume
    equals tk_fdk_device on the same input bit for bit."""
    import torch

    g = small_geometry(W=48, N=150, H=40, vol=(40, 40, 32))
    G = orc.geom_from(g)
    proj = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=3), G, "proj")  # [N][H][W]
    if layout == "sinogram":
        proj = np.ascontiguousarray(np.transpose(proj, (1, 0, 2)))
    fbp = FilteredBackProjection(raise_on_error=True)
    fbp.SetSinogramProperties(None, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau)
    fbp.SetReconstructionProperties(None, g.X, g.cx, g.Y, g.cy, g.Z, g.cz, g.rot)
    fbp.SetPrecision(prec)
    if raw:
        counts = counts_u16(proj, 60000.0, seed=4)
        fbp.SetProjectionsU16(counts, layout, flat_value=60000.0)
        d_in = torch.from_numpy(counts.view(np.int16)).cuda()
        ff, itype = device.flatfield(flat_value=60000.0), _lib.TK_INPUT_U16
    else:
        fbp.SetSinogramProperties(proj, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau)
        fbp.SetInputLayout(layout)
        d_in, ff, itype = torch.from_numpy(proj).cuda(), None, _lib.TK_INPUT_F32
    fbp.Initialize()
    vol = torch.empty((g.Z, g.Y, g.X), dtype=torch.float32, device="cuda")
    fbp.ReconstructToDevice(vol.data_ptr())
    fbp.close()
    ref = device.fdk_device(g, d_in, itype, _lib.LAYOUTS[layout], ff=ff, precision=_lib.PRECISIONS[prec])
    torch.cuda.synchronize()
    np.testing.assert_array_equal(vol.cpu().numpy(), ref.cpu().numpy())


def test_launch_count_and_fma_rate(cuda, case):
    """One FDK from uint16 counts with FP16 storage is three launches: the
    analytic storage scale, the fused filter and one backprojection."""
    import ctypes

    import torch

    g, G, ell, sino = case
    raw = counts_u16(np.transpose(sino, (1, 0, 2)), 60000.0, seed=2)
    d_in = to_dev(raw.view(np.int16), torch)
    ff = device.flatfield(flat_value=60000.0)
    L = _lib.load()
    device.fdk_device(g, d_in, _lib.TK_INPUT_U16, _lib.TK_LAYOUT_PROJECTION, ff=ff, precision=_lib.TK_F16)
    n0 = L.tk_kernel_launches()
    device.fdk_device(g, d_in, _lib.TK_INPUT_U16, _lib.TK_LAYOUT_PROJECTION, ff=ff, precision=_lib.TK_F16)
    assert L.tk_kernel_launches() - n0 == 3
    r = ctypes.c_double()
    _lib.check(L.tk_measure_fp32_fma_rate(ctypes.byref(r)))
    assert 10.0 < r.value < 200.0  # TFLOP/s


def test_full_size_1024_sampled_slices(orc, cuda):
    """The 720 x 1024^2 uint16 workload at full size: GPU vs FP64 oracle on
    sampled slices (the oracle filters only the detector rows they need)."""
    import torch
    from tomokvas_gb300.geometry import config

    g = config("c2")
    G = orc.geom_from(g)
    ell = random_ellipsoids(40, g.fov_radius_cm, g.Z * g.voxel_cm / 2, seed=11)
    line = device.phantom_project(g, ell, _lib.TK_LAYOUT_PROJECTION)  # [N][H][W]
    gen = torch.Generator(device="cuda").manual_seed(3)
    counts = torch.poisson(60000.0 * torch.exp(-line), generator=gen).clamp_(0, 65535)
    raw = counts.to(torch.int32).to(torch.int16)  # the bits of uint16 counts
    del line, counts
    ff = device.flatfield(flat_value=60000.0)
    raw_h = raw.cpu().numpy().view(np.uint16)
    sino = orc.log_u16(raw_h, np.float32(60000.0))  # [H][N][W]
    groups = [np.array([480, 512, 544], dtype=np.int32), np.array([1010], dtype=np.int32)]
    refs = [orc.fdk_f64(sino, G, "hann", zs) for zs in groups]  # one narrow row band each
    del sino
    rest = [orc.fdk_u16_f32_sampled(raw_h, G, 60000.0, window="hann", zlist=zs) for zs in groups]

    def grouped(vs):  # relative RMSE over all sampled slices together
        num = sum(float(np.sum((v - r) ** 2)) for v, r in zip(vs, refs))
        return (num / sum(float(np.sum(r ** 2)) for r in refs)) ** 0.5

    rest_err = grouped(rest)
    for prec, tol in [(_lib.TK_F32, noisy_tol(rest_err)), (_lib.TK_F32_COEF, noisy_tol(rest_err)),
                      (_lib.TK_F16, F16_RMSE)]:
        vol = device.fdk_device(g, raw, _lib.TK_INPUT_U16, _lib.TK_LAYOUT_PROJECTION, ff=ff,
                                window=_lib.TK_WINDOW_HANN, precision=prec)
        torch.cuda.synchronize()
        got = [vol[torch.from_numpy(zs).long().cuda()].cpu().numpy() for zs in groups]
        del vol
        assert grouped(got) < tol, (prec, grouped(got), rest_err)
    assert device.device_error_flags() == 0


def _handle_run(g, data, layout, prec, pipeline, zb, counts=None, after_init=None, window=None):
    out = VolumeSink(g.X, g.Y, g.Z, zb)
    fbp = FilteredBackProjection(raise_on_error=True)
    fbp.SetBlockSize(zb)
    fbp.SetPipeline(pipeline)
    fbp.SetSinogramProperties(data, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau)
    fbp.SetReconstructionProperties(out, g.X, g.cx, g.Y, g.cy, g.Z, g.cz, g.rot)
    fbp.SetScaleXYZ(g.scale)
    fbp.SetPrecision(prec)
    if window:
        fbp.SetFilter(window)
    if counts is not None:
        fbp.SetProjectionsU16(counts, layout, flat_value=60000.0)
    else:
        fbp.SetInputLayout(layout)
    L = _lib.load()
    n0 = L.tk_kernel_launches()
    fbp.Initialize()
    if after_init:
        after_init(fbp)
    fbp.CalculateReconstruction()
    launches = L.tk_kernel_launches() - n0
    fbp.close()
    return out, launches


def pipelined_launches(g, nblk, last_slices, zoff=None, quad=False, layout="projection"):
    """Launches of a pipelined Initialize (tk_fdk_initialize).  Chunks of
    max(32, ceil(N/8)) angles, each a storage-scale and a filter launch; the
    chunks ending by the first quarter of the angles backprojected block by
    block, or in one launch over all blocks when the blocks' slice
    coordinates are those of one launch (float32 arithmetic) and the blocks
    start on 64-slice boundaries; one launch per block over the rest, the
    last block in two when it holds at least 128 slices.  With the
    quarter-turn kernel (quad): C chunks (the first of 8, 6, 5, 4, 3 that
    divides N/4) of four N/(4C)-angle ranges a quarter turn apart, each chunk
    (detector frames) or each range (sinograms) a storage-scale and a filter
    launch; the first (C + 2) // 4 chunks
    backprojected together once filtered (one launch, or one per block when
    not merged), the rest per block as above."""
    split = 1 if (last_slices // 2) // 64 * 64 > 0 else 0
    merged = False
    if zoff is not None and g.zb % 64 == 0:
        f = np.float32
        merged = all(f(z) + f(zoff[n]) == f(n * g.zb + z) + f(zoff[0])
                     for n in range(nblk) for z in range(min(g.zb, g.Z - n * g.zb)))
    if quad:
        C = next(c for c in (8, 6, 5, 4, 3) if (g.N // 4) % c == 0)
        return (2 if layout == "projection" else 8) * C + (1 if merged else nblk) + nblk + split
    chunk = max(32, -(-g.N // 8))
    nch = -(-g.N // chunk)
    major_end = min(g.N - chunk, chunk * max(1, (nch + 2) // 4))
    major = sum(1 for b0 in range(0, g.N, chunk) if b0 + min(chunk, g.N - b0) <= major_end)
    return 2 * nch + major * (1 if merged else nblk) + nblk + split


@pytest.mark.parametrize("vol_shape,zb,prec,raw,layout", [
    ((40, 40, 40), 16, "f32", False, "projection"),   # blocks 16, 16, 8
    ((40, 40, 33), 16, "f16", True, "projection"),    # last-slice quirk
    ((36, 40, 30), 64, "f32c", False, "projection"),  # one block, zb > Z
    ((40, 40, 128), 128, "f16", True, "projection"),  # the last block's launch split at 64 slices
    ((40, 40, 256), 128, "f16", True, "projection"),  # two blocks: first quarter in one launch
    ((40, 40, 40), 16, "f16", True, "sinogram"),      # [H][N][W], packed per chunk by strided copies
    ((40, 40, 33), 16, "f32", False, "sinogram"),
    ((64, 64, 128), 128, "f16", True, "projection"),  # quarter-turn kernel: 5 chunks of 4 x 15 angles
    ((64, 64, 256), 128, "f16", True, "projection"),  # quarter-turn, first chunk in one launch
    ((64, 64, 40), 16, "f16", True, "sinogram")])     # quarter-turn, blocks on two streams
def test_pipelined_handle_equals_regular(orc, cuda, vol_shape, zb, prec, raw, layout):
    """tk_fdk_set_pipeline: Initialize uploads N = 300 projections in 38-angle
    chunks, filters each as it lands, backprojects the chunks of the first
    76 angles into the whole volume with the Z-block schedule as they land,
    then each block over the other 224 angles; CalculateReconstruction only
    delivers blocks.  The volume equals the regular path's to FP32 rounding of
    the partial sums, with the same blocks requested, the same last-slice
    quirk, and the launches of that schedule.  Square 64-voxel FP16 volumes
    take the quarter-turn schedule: 5 chunks of four 15-angle ranges a quarter
    turn apart, filtered on their own stream, the first backprojected once
    filtered."""
    g = small_geometry(W=48, N=300, H=48, vol=vol_shape, zb=zb)
    G = orc.geom_from(g)
    proj = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=5), G, "proj")  # [N][H][W]
    if layout == "sinogram":
        proj = np.ascontiguousarray(np.transpose(proj, (1, 0, 2)))
    counts = counts_u16(proj, 60000.0, seed=6) if raw else None
    data = None if raw else proj
    reg, _ = _handle_run(g, data, layout, prec, False, zb, counts)
    pip, launches = _handle_run(g, data, layout, prec, True, zb, counts)
    zoff = orc.zblocks(G)
    nblk = len(zoff)
    last = g.Z - (nblk - 1) * zb if nblk * zb > g.Z else zb
    quad = prec == "f16" and vol_shape[0] == vol_shape[1] == 64
    assert launches == pipelined_launches(g, nblk, last, zoff, quad, layout)
    assert pip.blocks_requested == reg.blocks_requested
    assert rel_rmse(pip.volume, reg.volume) < 1e-6
    assert max_abs(pip.volume, reg.volume) < 1e-5 * np.abs(reg.volume).max()
    if (g.Z - 1) % zb == 0:
        assert np.all(pip.volume[-1] == 0) and np.all(reg.volume[-1] == 0)
    if not raw:  # the FP32 restatement follows the handle's Z-block schedule (last-slice quirk included)
        sino = proj if layout == "sinogram" else np.ascontiguousarray(np.transpose(proj, (1, 0, 2)))
        assert rel_rmse(pip.volume, orc.fdk_f32(sino, G)) < (F16_RMSE if prec == "f16" else F32_RMSE)


@pytest.mark.parametrize("vol_shape,prec,raw", [((40, 40, 40), "f32", False),
                                               ((64, 64, 40), "f16", True)])  # quarter-turn chunks
def test_setter_after_pipelined_initialize(orc, cuda, vol_shape, prec, raw):
    """A setter after Initialize (here the window) drops the pipelined volume
    and the filtered projections: the sinogram, stored on the device as
    per-chunk [H][nb][W] blocks (for the quarter-turn schedule, blocks of the
    four ranges of each chunk), is unpacked and filtered again, and the
    volume equals a fresh regular run with that window."""
    g = small_geometry(W=48, N=300, H=48, vol=vol_shape, zb=16)
    G = orc.geom_from(g)
    sino = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=7), G, "sino")
    counts = counts_u16(sino, 60000.0, seed=8) if raw else None
    data = None if raw else sino
    hann = lambda fbp: fbp.SetFilter("hann")  # noqa: E731
    changed, launches = _handle_run(g, data, "sinogram", prec, True, 16, counts, after_init=hann)
    fresh, _ = _handle_run(g, data, "sinogram", prec, False, 16, counts, window="hann")
    zoff = orc.zblocks(G)
    nblk = len(zoff)
    # the pipelined pass, then a regular one
    assert launches == pipelined_launches(g, nblk, g.Z - (nblk - 1) * 16, zoff, raw, "sinogram") + 2 + nblk
    # the fresh run filters in even 64-angle chunks, which pair FFT rows as one pass does
    assert rel_rmse(changed.volume, fresh.volume) < 1e-7
    assert max_abs(changed.volume, fresh.volume) <= 1e-6 * np.abs(fresh.volume).max()
