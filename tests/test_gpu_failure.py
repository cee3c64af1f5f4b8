"""The failure reporting of the kernels, exercised without a GPU fault.

* A wait that runs out: tk_diag_wait_timeout launches a CTA that waits, with
  the library's bounded mbarrier wait and a 1 ms limit, on a barrier armed for
  copies that are never issued; the kernel returns and leaves ERR_WAIT_TIMEOUT
  in the device error word, and the context stays usable.
* A staged box too small for the footprint: tk_diag_shrink_box takes rows off
  every backprojection's box; the kernels' bounds checks skip the reads that
  would fall outside, set ERR_BOX_OVERFLOW, and the FilteredBackProjection
  handle returns TK_ERR_DEVICE.  With the box restored, the same run is clean
  and equals the run before.
"""
import numpy as np
import pytest

from _util import small_geometry
from tomokvas_gb300 import _lib, device
from tomokvas_gb300.fbp import FilteredBackProjection, VolumeSink
from tomokvas_gb300.phantom import head_phantom

pytestmark = pytest.mark.gpu

ERR_BOX_OVERFLOW, ERR_WAIT_TIMEOUT = 0x1, 0x2


def test_bounded_wait_reports_timeout(cuda):
    import torch

    L = _lib.load()
    assert device.device_error_flags() == 0
    _lib.check(L.tk_diag_wait_timeout(1.0, None))
    torch.cuda.synchronize()
    assert device.device_error_flags() == ERR_WAIT_TIMEOUT  # read and cleared
    assert device.device_error_flags() == 0
    assert L.tk_diag_wait_timeout(0.0, None) == _lib.TK_ERR_INVALID
    x = torch.ones(1024, device="cuda")  # the context still runs work
    assert float(x.sum().item()) == 1024.0


def handle_run(g, sino, prec):
    sink = VolumeSink(g.X, g.Y, g.Z, g.zb)
    fbp = FilteredBackProjection(raise_on_error=False)
    try:
        fbp.SetBlockSize(g.zb)
        fbp.SetSinogramProperties(sino, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau)
        fbp.SetReconstructionProperties(sink, g.X, g.cx, g.Y, g.cy, g.Z, g.cz, g.rot)
        fbp.SetScaleXYZ(g.scale)
        fbp.SetPrecision(prec)
        assert fbp.Initialize() == 0
        rc = fbp.CalculateReconstruction()
    finally:
        fbp.close()
    return rc, sink.volume.copy()


@pytest.mark.parametrize("prec", ["f16", "f32"])  # the quarter-turn kernel; the direct FP32 walk
def test_box_overflow_is_reported(orc, cuda, prec):
    L = _lib.load()
    g = small_geometry(W=64, N=60, H=64, vol=(64, 64, 40), zb=16)
    G = orc.geom_from(g)
    sino = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=8), G, "sino")
    rc0, v0 = handle_run(g, sino, prec)
    assert rc0 == 0 and device.device_error_flags() == 0
    try:
        _lib.check(L.tk_diag_shrink_box(1 << 20))  # boxes of one row
        rc1, _ = handle_run(g, sino, prec)
    finally:
        _lib.check(L.tk_diag_shrink_box(0))
    assert rc1 == _lib.TK_ERR_DEVICE
    assert b"self-check" in L.tk_last_error()
    assert device.device_error_flags() == 0  # the handle read and cleared the word
    rc2, v2 = handle_run(g, sino, prec)
    assert rc2 == 0 and device.device_error_flags() == 0
    np.testing.assert_array_equal(v2, v0)
