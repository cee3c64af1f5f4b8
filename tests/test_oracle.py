"""CPU oracle: closed-form pins of the reference's construction and quirks.

The reference (Lukas-kV/TomoKvas) ships no tests or fixtures, so the oracle
is pinned by identities that the reference's own code implies:
  * its FFT filter (kernel.cu:557-802) equals a linear convolution with the
    zero-phase truncated Ram-Lak kernel tau*RamLak(n)/2 when W = 0 mod 4;
  * its Z-block schedule (kernel.cu:398-400, 821) places slice z at
    aZ = scale*(z - (Z-1)/2 - cz), and drops the last slice when (Z-1) % ZB == 0;
  * axis flips (kernel.cu:86-88) mirror the volume;
plus FP32-vs-FP64 agreement and reconstruction of an analytic phantom.
"""
import math

import numpy as np
import pytest

from _util import max_abs, rel_rmse, small_geometry
from tomokvas_gb300.phantom import counts_u16, head_phantom


def ramlak(n, tau):
    if n == 0:
        return 1.0 / (4.0 * tau * tau)
    if n % 2 == 0:
        return 0.0
    return -1.0 / (n * n * math.pi * math.pi * tau * tau)


@pytest.mark.parametrize("W,p", [(1, 4), (2, 4), (3, 8), (256, 512), (768, 2048), (1024, 2048), (2048, 4096)])
def test_pad_length(orc, W, p):
    # kernel.cu:570-573
    assert orc.pad_length(W) == p


@pytest.mark.parametrize("W", [64, 256, 1024])
def test_filter_equals_truncated_ramlak(orc, W):
    tau = 0.02
    k, p = orc.filter_kernel(W, tau, "ramlak")
    exp = np.zeros(2 * W - 1)
    for n in range(-(W // 2 - 1), W // 2):
        # taps are float (FillFilter), computed in double from the float pitch
        exp[n + W - 1] = tau * float(np.float32(ramlak(n, float(np.float32(tau))))) / 2.0
    assert np.max(np.abs(k - exp)) <= 1e-9 * np.max(np.abs(exp))


def test_filter_w2mod4_is_symmetric_and_not_truncated(orc):
    W, tau = 66, 0.05
    k, _ = orc.filter_kernel(W, tau, "ramlak")
    assert np.allclose(k, k[::-1], rtol=0, atol=1e-12 * np.max(np.abs(k)))
    # |FFT(h)| makes it differ from the truncated Ram-Lak at W = 2 mod 4
    assert abs(k[W - 1 + 2]) > 1e-8 * abs(k[W - 1])


@pytest.mark.parametrize("window", ["ramlak", "shepp_logan", "hann"])
def test_filter_stage_f32_matches_f64(orc, window):
    g = small_geometry(W=96, N=16, H=8, vol=(8, 8, 8))
    G = orc.geom_from(g)
    rng = np.random.default_rng(3)
    sino = rng.normal(size=(g.H, g.N, g.W)).astype(np.float32)
    w = orc.weight_f32(sino, G)
    q32 = orc.filter_f32(w, G, window) / orc.pad_length(g.W)
    q64 = orc.weight_filter_f64(sino, G, window)
    assert rel_rmse(q32, q64) < 2e-6


def test_filter_delta_response_is_kernel(orc):
    g = small_geometry(W=64, N=1, H=1, vol=(8, 8, 8))
    g = g.replace(D=1e9)  # cosine weight -> 1
    G = orc.geom_from(g)
    sino = np.zeros((1, 1, 64), dtype=np.float32)
    sino[0, 0, 20] = 1.0
    q = orc.weight_filter_f64(sino, G, "hann")[0, 0]
    k, _ = orc.filter_kernel(64, float(np.float32(g.tau)), "hann")  # the geometry carries tau as float
    assert np.allclose(q, k[63 - 20:63 - 20 + 64], rtol=0, atol=1e-12 * np.abs(k).max())


@pytest.mark.parametrize("Z,zb,exact", [(256, 16, True), (255, 30, False), (1024, 30, False), (64, 7, True),
                                         (65, 16, True)])
def test_zblock_centring(orc, Z, zb, exact):
    # dcorZ = (nblocks - nr_Z) * ZB / 2 is rounded in float (kernel.cu:398-400), so the
    # reference's slices sit within ~1e-5 voxel of z - (Z-1)/2, exactly only when
    # (Z-1)/ZB is representable.
    g = small_geometry(vol=(8, 8, Z), zb=zb)
    G = orc.geom_from(g)
    zoff = orc.zblocks(G)
    assert len(zoff) == math.ceil(np.float32(Z - 1) / np.float32(zb))
    dev = []
    for n, off in enumerate(zoff):
        for zl in range(zb):
            z = n * zb + zl
            dev.append(abs(float(np.float32(zl) + off) - (z - (Z - 1) / 2.0)))
    assert max(dev) < 1e-4
    assert (max(dev) == 0.0) == exact


def test_last_slice_quirk(orc):
    # (Z-1) % ZB == 0: the reference never computes the last slice (kernel.cu:398-399, 819)
    g = small_geometry(W=32, N=24, H=48, vol=(16, 16, 33), zb=16)
    G = orc.geom_from(g)
    sino = np.ones((g.H, g.N, g.W), dtype=np.float32)
    q = orc.filter_f32(orc.weight_f32(sino, G), G)
    vol = orc.bp_f32(q, G)
    assert len(orc.zblocks(G)) == 2
    assert np.all(vol[32] == 0) and np.any(vol[31] != 0) and np.any(vol[0] != 0)
    G2 = orc.geom_from(g.replace(Z=34))
    vol2 = orc.bp_f32(orc.filter_f32(orc.weight_f32(sino, G2), G2), G2)
    assert np.any(vol2[33] != 0)


@pytest.fixture(scope="module")
def phantom_case(orc):
    g = small_geometry()
    G = orc.geom_from(g)
    ell = head_phantom(g.fov_radius_cm * 0.9, seed=1)
    sino = orc.project_ellipsoids(ell, G, "sino")
    return g, G, ell, sino


def test_fdk_reconstructs_phantom(orc, phantom_case):
    g, G, ell, sino = phantom_case
    z = np.array([g.Z // 2 - 5, g.Z // 2, g.Z // 2 + 5], dtype=np.int32)
    rec = orc.fdk_f64(sino, G, "ramlak", z)
    truth = orc.voxelise_ellipsoids(ell, G, z)
    # interior of the flat regions: away from edges (truth constant in a 3x3 neighbourhood)
    t = truth[1]
    flat = np.ones_like(t, dtype=bool)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            flat &= np.roll(np.roll(t, dy, 0), dx, 1) == t
    flat &= t > 0.1
    assert flat.sum() > 200
    assert np.sqrt(np.mean((rec[1] - t)[flat] ** 2)) < 0.03 * t.max()


def test_fdk_f32_matches_f64(orc, phantom_case):
    g, G, ell, sino = phantom_case
    v32 = orc.fdk_f32(sino, G)
    v64 = orc.fdk_f64(sino, G)
    assert rel_rmse(v32, v64) < 1e-5
    assert max_abs(v32, v64) < 1e-4 * np.abs(v64).max()


def test_axis_flip_mirrors_volume(orc, phantom_case):
    g, G, ell, sino = phantom_case
    v = orc.fdk_f32(sino, G)
    Gf = orc.geom_from(g.replace(dirx=1))
    vf = orc.fdk_f32(sino, Gf)
    assert np.array_equal(vf, v[:, :, ::-1])


def test_log_transform(orc):
    rng = np.random.default_rng(0)
    raw = rng.integers(0, 60000, size=(3, 4, 5)).astype(np.uint16)
    flat = np.full((4, 5), 60000.0, dtype=np.float32)
    dark = np.full((4, 5), 100.0, dtype=np.float32)
    out = orc.log_u16(raw, flat, dark, A=1.5, B=0.25, invert=True, floor_counts=0.5)
    num = np.maximum(raw.astype(np.float64) - 100.0, 0.5)
    ref = -(1.5 * np.log(num / (60000.0 - 100.0)) + 0.25)
    assert np.allclose(out, np.transpose(ref, (1, 0, 2)).astype(np.float32), rtol=1e-6, atol=1e-6)


def test_u16_counts_roundtrip(orc, phantom_case):
    g, G, ell, sino = phantom_case
    raw = counts_u16(np.transpose(sino, (1, 0, 2)), 60000.0, seed=2)
    p = orc.log_u16(raw, np.float32(60000.0))
    # Poisson noise at I0 = 60000 is small relative to the line integrals
    assert np.sqrt(np.mean((p - sino) ** 2)) < 0.02


def test_fp64_adjoint_is_exact_transpose(orc):
    """<A x, y> = <x, A^T y> for the FP64 FDK and its FP64 adjoint."""
    g = small_geometry(W=48, N=40, H=40, vol=(32, 32, 32), rot=0.2, dirx=1)
    G = orc.geom_from(g)
    rng = np.random.default_rng(0)
    x = rng.normal(size=(g.H, g.N, g.W)).astype(np.float32)
    y = rng.normal(size=(g.Z, g.Y, g.X)).astype(np.float32)
    for window in ("ramlak", "hann"):
        lhs = float(np.sum(orc.fdk_f64(x, G, window) * y))
        rhs = float(np.sum(x.astype(np.float64) * orc.fdk_adjoint_f64(y, G, window)))
        assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_oracle_backprojection_pair_is_a_transpose(orc):
    """<B q, x> = <q, B^T x> in FP64 for the refinement's pair (orc_b_f64, orc_bt_f64), with a flip and a rotation."""
    g = small_geometry(W=24, N=10, H=20, vol=(16, 14, 12), dirx=1, rot=0.4)
    G = orc.geom_from(g)
    rng = np.random.default_rng(2)
    q = rng.normal(size=(g.N, g.H, g.W))
    x = rng.normal(size=(g.Z, g.Y, g.X))
    lhs = float(np.sum(orc.b_f64(q, G) * x))
    rhs = float(np.sum(q * orc.bt_f64(x, G)))
    assert abs(lhs - rhs) < 1e-12 * max(abs(lhs), 1.0)
