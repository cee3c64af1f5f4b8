"""Pins against the reference itself: golden outputs of Lukas-kV/TomoKvas's own
FDK kernels (FBPG/kernel.cu + cuFFT on a GB300, tests/golden/make_golden.py).

CPU: the oracle's FP32 restatement and FP64 FDK against the reference.
GPU: the CUDA path, through the FilteredBackProjection mirror with the same
Z-block schedule, against the reference.
"""
import glob
import os

import numpy as np
import pytest

from _util import max_abs, rel_rmse
from tomokvas_gb300.geometry import FDKGeometry

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_*.npz")))
INT_FIELDS = {"W", "N", "H", "X", "Y", "Z", "dirx", "diry", "dirz", "zb"}


def load(path):
    d = np.load(path)
    kw = {}
    for f, v in zip(d["fields"], d["geometry"]):
        f = str(f)
        kw[f] = int(v) if f in INT_FIELDS else float(v)
    return FDKGeometry(**kw), d


@pytest.fixture(scope="module", params=GOLDEN, ids=[os.path.basename(p)[4:-4] for p in GOLDEN])
def golden(request, orc):
    g, d = load(request.param)
    G = orc.geom_from(g)
    sino = orc.project_ellipsoids(d["ellipsoids"], G, "sino")
    chk = np.array([np.sum(sino, dtype=np.float64), np.sum(np.square(sino, dtype=np.float64))])
    assert np.allclose(chk, d["sino_checksum"], rtol=1e-6), "regenerated projections differ from the reference's"
    return g, G, sino, d["slices"], d["volume"]


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 5


def test_oracle_f32_matches_reference(orc, golden):
    # same operation order; the FP32 FFT is the oracle's own instead of cuFFT
    g, G, sino, z, ref = golden
    v = orc.fdk_f32(sino, G, "ramlak", z)
    assert rel_rmse(v, ref) < 5e-6
    assert max_abs(v, ref) < 5e-5 * np.abs(ref).max()


def test_oracle_f64_matches_reference(orc, golden):
    g, G, sino, z, ref = golden
    # the FP64 oracle centres slices exactly; the reference's float dcorZ shifts them by ~1e-5 voxel
    v = orc.fdk_f64(sino, G, "ramlak", z)
    assert rel_rmse(v, ref) < 1e-5


def test_reference_drops_last_slice_when_z_minus_1_divides(golden):
    g, G, sino, z, ref = golden
    if (g.Z - 1) % g.zb == 0 and (g.Z - 1) in list(z):
        assert np.all(ref[list(z).index(g.Z - 1)] == 0)


@pytest.mark.gpu
def test_cuda_path_matches_reference(orc, cuda, golden):
    from tomokvas_gb300.fbp import FilteredBackProjection, VolumeSink

    g, G, sino, z, ref = golden
    out = VolumeSink(g.X, g.Y, g.Z, g.zb)
    fbp = FilteredBackProjection(raise_on_error=True)
    fbp.SetBlockSize(g.zb)
    fbp.SetAxisDirection(bool(g.dirx), bool(g.diry), bool(g.dirz))
    fbp.SetSinogramProperties(sino, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau)
    fbp.SetReconstructionProperties(out, g.X, g.cx, g.Y, g.cy, g.Z, g.cz, g.rot)
    fbp.SetScaleXYZ(g.scale)
    fbp.Initialize()
    fbp.CalculateReconstruction()
    fbp.close()
    v = out.volume[z]
    assert rel_rmse(v, ref) < 1e-5
    assert max_abs(v, ref) < 1e-4 * np.abs(ref).max()


@pytest.mark.gpu
def test_cuda_f16_path_matches_reference(orc, cuda, golden):
    """FP16 coefficient storage (the default form) against the reference's own
    outputs: within the FP16-storage bound.  On the square, centred,
    unflipped fixtures with N divisible by 4 this runs the quarter-turn
    backprojector, elsewhere the general FP16 walk."""
    from tomokvas_gb300.fbp import FilteredBackProjection, VolumeSink

    g, G, sino, z, ref = golden
    out = VolumeSink(g.X, g.Y, g.Z, g.zb)
    fbp = FilteredBackProjection(raise_on_error=True)
    fbp.SetBlockSize(g.zb)
    fbp.SetAxisDirection(bool(g.dirx), bool(g.diry), bool(g.dirz))
    fbp.SetSinogramProperties(sino, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau)
    fbp.SetReconstructionProperties(out, g.X, g.cx, g.Y, g.cy, g.Z, g.cz, g.rot)
    fbp.SetScaleXYZ(g.scale)
    fbp.SetPrecision("f16")
    fbp.Initialize()
    fbp.CalculateReconstruction()
    fbp.close()
    assert rel_rmse(out.volume[z], ref) < 5e-4
