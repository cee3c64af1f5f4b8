"""Volume data-consistency refinement (tk_refine_*): gradient steps
x <- x - alpha B (B^T x - q) on L(x) = ||B^T x - q||^2 from the FDK volume,
with the filtered projections q checkpointed as FP32 or FP16 samples.

Bounds:
  one step against the FP64 oracle step (orc_b_f64 / orc_bt_f64 on the same
  x0 and q): the update x1 - x0 within 1e-4 relative RMSE (FP32 arithmetic,
  shared-memory atomics in B^T), the loss within 1e-5;
  20 steps: the loss falls at every step, by at least 10 %;
  FP16 checkpoint: the volume after 5 steps within 1e-3 of the FP32
  checkpoint's (FP16 rounding of q, 2^-11 relative per sample).
"""
import ctypes

import numpy as np
import pytest

from _util import rel_rmse, small_geometry
from tomokvas_gb300 import _lib, device
from tomokvas_gb300.phantom import head_phantom

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problem(orc, cuda):
    import torch

    g = small_geometry(W=64, N=60, H=64, vol=(48, 48, 40))
    G = orc.geom_from(g)
    sino = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=17), G, "sino")
    rng = np.random.default_rng(5)
    sino = (sino + 0.01 * np.abs(sino).max() * rng.normal(size=sino.shape)).astype(np.float32)
    d = torch.from_numpy(sino).cuda()
    x0 = device.fdk_device(g, d, precision=_lib.TK_F32)
    ws = device.refine_workspace(g)
    return g, G, d, x0, ws


def test_refine_step_matches_fp64_oracle(orc, problem):
    import torch

    g, G, d, x0, ws = problem
    ckpt = device.refine_checkpoint(g, d, workspace=ws)
    alpha = device.refine_step_size(g, iters=6, workspace=ws)
    assert alpha > 0
    x = x0.clone()
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    device.refine_volume(g, ckpt, x, alpha, 1, loss=loss, workspace=ws)
    torch.cuda.synchronize()
    assert device.device_error_flags() == 0
    x0h = x0.cpu().numpy().astype(np.float64)
    q = ckpt.cpu().numpy()[:, :, :g.W].astype(np.float64)
    r = orc.bt_f64(x0h, G) - q
    x1_ref = x0h - alpha * orc.b_f64(r, G)
    x1 = x.cpu().numpy().astype(np.float64)
    assert rel_rmse(x1 - x0h, x1_ref - x0h) < 1e-4
    assert abs(float(loss.item()) - float(np.sum(r * r))) < 1e-5 * float(np.sum(r * r))


def test_refine_loss_falls_every_step(problem):
    import torch

    g, G, d, x0, ws = problem
    ckpt = device.refine_checkpoint(g, d, workspace=ws)
    alpha = device.refine_step_size(g, iters=6, workspace=ws)
    x = x0.clone()
    loss = torch.zeros(20, dtype=torch.float64, device="cuda")
    device.refine_volume(g, ckpt, x, alpha, 20, loss=loss, workspace=ws)
    torch.cuda.synchronize()
    ls = loss.cpu().numpy()
    assert device.device_error_flags() == 0
    assert np.all(np.diff(ls) < 0), ls
    assert ls[-1] < 0.9 * ls[0], ls


def test_refine_fp16_checkpoint(problem):
    import torch

    g, G, d, x0, ws = problem
    c32 = device.refine_checkpoint(g, d, precision=_lib.TK_F32, workspace=ws)
    c16 = device.refine_checkpoint(g, d, precision=_lib.TK_F16, workspace=ws)
    assert c16.dtype == torch.float16 and c16.numel() == c32.numel()
    assert rel_rmse(c16.float().cpu().numpy(), c32.cpu().numpy()) < 1e-3
    alpha = device.refine_step_size(g, iters=6, workspace=ws)
    xa, xb = x0.clone(), x0.clone()
    device.refine_volume(g, c32, xa, alpha, 5, workspace=ws)
    device.refine_volume(g, c16, xb, alpha, 5, workspace=ws)
    torch.cuda.synchronize()
    assert device.device_error_flags() == 0
    assert rel_rmse(xb.cpu().numpy(), xa.cpu().numpy()) < 1e-3


def test_refine_rejects_bad_arguments(problem):
    g, G, d, x0, ws = problem
    L = _lib.load()
    gc = _lib.Geometry(**{k: getattr(g, k) for k, _ in _lib.Geometry._fields_})
    args = (ctypes.byref(gc), ws.data_ptr())
    assert L.tk_refine_volume(*args, _lib.TK_BF16, 1.0, 1, x0.data_ptr(), None, ws.data_ptr(), ws.numel(),
                              None) == _lib.TK_ERR_INVALID
    assert L.tk_refine_volume(*args, _lib.TK_F32, -1.0, 1, x0.data_ptr(), None, ws.data_ptr(), ws.numel(),
                              None) == _lib.TK_ERR_INVALID
    assert L.tk_refine_volume(*args, _lib.TK_F32, 1.0, 1, x0.data_ptr(), None, ws.data_ptr(), 16,
                              None) == _lib.TK_ERR_INVALID
