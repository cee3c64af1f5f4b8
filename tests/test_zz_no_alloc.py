"""tk_fdk_device_noalloc: the whole-FDK entry point for callers that cannot
allocate device memory (a fixed memory budget reserved at start-up, or a
callback / timing-critical loop where cudaMalloc's implicit synchronisation
and possible failure are not acceptable).  It must give the same volume as
tk_fdk_device, whose workspace the caller allocates, on consecutive calls
that reuse its static scratch array.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

from _util import rel_rmse, small_geometry
from tomokvas_gb300 import _lib, device
from tomokvas_gb300.phantom import head_phantom

pytestmark = pytest.mark.gpu

F32_RMSE = 1e-5  # the FP32 tolerance of the parity tests


def test_noalloc_matches_workspace_entry_point(orc, cuda):
    import torch

    L = _lib.load()
    g = small_geometry(W=64, N=90, H=64, vol=(48, 48, 40))
    G = orc.geom_from(g)
    sino = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=12), G, "sino")
    d_in = torch.from_numpy(sino).cuda()
    gc = g.to_c()
    stream = torch.cuda.current_stream().cuda_stream
    for prec in (_lib.TK_F32, _lib.TK_F16):
        ref = device.fdk_device(g, d_in, precision=prec).cpu().numpy()  # caller-allocated workspace
        for call in range(2):  # the second call reuses the scratch the first one left behind
            vol = torch.full((g.Z, g.Y, g.X), float("nan"), dtype=torch.float32, device="cuda")
            rc = L.tk_fdk_device_noalloc(ctypes.byref(gc), d_in.data_ptr(), _lib.TK_INPUT_F32,
                                         _lib.TK_LAYOUT_SINOGRAM, None, _lib.TK_WINDOW_RAMLAK, prec,
                                         vol.data_ptr(), stream)
            assert rc == _lib.TK_OK, L.tk_last_error()
            torch.cuda.synchronize()
            got = vol.cpu().numpy()
            assert np.isfinite(got).all()
            assert rel_rmse(got, ref) <= F32_RMSE, (prec, call)
        # a warmed-up call takes no device memory: the free bytes do not move across one more call
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        rc = L.tk_fdk_device_noalloc(ctypes.byref(gc), d_in.data_ptr(), _lib.TK_INPUT_F32, _lib.TK_LAYOUT_SINOGRAM,
                                     None, _lib.TK_WINDOW_RAMLAK, prec, vol.data_ptr(), stream)
        torch.cuda.synchronize()
        assert rc == _lib.TK_OK and torch.cuda.mem_get_info()[0] == free0
    assert device.device_error_flags() == 0


def test_noalloc_rejects_problems_beyond_its_scratch(cuda):
    import torch

    L = _lib.load()
    g = small_geometry(W=1024, N=720, H=1024, vol=(16, 16, 16))  # 3 GB of FP32 filtered projections
    gc = g.to_c()
    rc = L.tk_fdk_device_noalloc(ctypes.byref(gc), ctypes.c_void_p(256), _lib.TK_INPUT_F32, _lib.TK_LAYOUT_SINOGRAM,
                                 None, _lib.TK_WINDOW_RAMLAK, _lib.TK_F32, ctypes.c_void_p(256),
                                 torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.TK_ERR_UNSUPPORTED
    assert b"static scratch" in L.tk_last_error()
