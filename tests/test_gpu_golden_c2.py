"""The headline workload against the reference's own output: 1024^3 from
720 x 1024^2 projections, the reference's FBPG/kernel.cu FDK (Ram-Lak, cuFFT,
Z blocks of 16) run on a GB300 by tests/golden/make_golden.py --c2, five
slices stored at every 4th voxel (tests/golden/c2ref_1024.npz).

The projections are regenerated by the same GPU projector that made them and
checked against the stored checksum.  Our path runs through the
FilteredBackProjection mirror with the same Z-block schedule.  The fixture
also holds the FP64 oracle on the same voxels: the reference's own FP32
pipeline (cuFFT filter, ceil-based lerps) sits about 1.5e-5 from it at this
size, so our FP32 path is held to the triangle bound (its own distance to
FP64 plus the reference's, at least 1e-5) against the reference, and to 1e-5
against FP64.  FP16 storage with FP32 interpolation (the chosen form): 5e-4
against both.  Relative RMSE over the stored voxels.
"""
import os

import numpy as np
import pytest

from _util import max_abs, rel_rmse
from tomokvas_gb300 import _lib, device
from tomokvas_gb300.fbp import FilteredBackProjection, VolumeSink
from tomokvas_gb300.geometry import FDKGeometry

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c2ref_1024.npz")
INT_FIELDS = {"W", "N", "H", "X", "Y", "Z", "dirx", "diry", "dirz", "zb"}


@pytest.fixture(scope="module")
def c2(cuda):
    if not os.path.exists(FIXTURE):
        pytest.skip("c2ref_1024.npz not generated")
    d = np.load(FIXTURE)
    kw = {str(f): (int(v) if str(f) in INT_FIELDS else float(v)) for f, v in zip(d["fields"], d["geometry"])}
    g = FDKGeometry(**kw)
    sino = device.phantom_project(g, d["ellipsoids"], _lib.TK_LAYOUT_SINOGRAM).cpu().numpy()
    chk = np.array([np.sum(sino, dtype=np.float64), np.sum(np.square(sino, dtype=np.float64))])
    assert np.allclose(chk, d["sino_checksum"], rtol=1e-9), "regenerated projections differ from the reference's"
    return g, sino, d["slices"], int(d["step"]), d["volume"], d["fp64"]


@pytest.mark.parametrize("prec,bound", [("f32", 1e-5), ("f16", 5e-4)])
def test_c2_against_reference_output(c2, prec, bound):
    g, sino, z, step, ref, f64 = c2
    sink = VolumeSink(g.X, g.Y, g.Z, g.zb)
    fbp = FilteredBackProjection(raise_on_error=True)
    try:
        fbp.SetBlockSize(g.zb)
        fbp.SetSinogramProperties(sino, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau)
        fbp.SetReconstructionProperties(sink, g.X, g.cx, g.Y, g.cy, g.Z, g.cz, g.rot)
        fbp.SetScaleXYZ(g.scale)
        fbp.SetPrecision(prec)
        fbp.Initialize()
        fbp.CalculateReconstruction()
    finally:
        fbp.close()
    got = np.ascontiguousarray(sink.volume[z][:, ::step, ::step])
    assert device.device_error_flags() == 0
    ours_f64, ref_f64 = rel_rmse(got, f64), rel_rmse(ref, f64)
    assert ref_f64 < 1e-4  # the fixture: the reference's FP32 FDK against FP64
    assert ours_f64 < bound
    assert rel_rmse(got, ref) < max(bound, ours_f64 + ref_f64)
    assert max_abs(got, ref) < 1e-3 * np.abs(ref).max()
