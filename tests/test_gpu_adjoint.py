"""Adjoint pair on the GPU: tk_fdk_forward (A) and tk_fdk_backward (A^T).

A maps line integrals to the volume (cosine weight, ramp filter,
backprojection); A^T is built from the transposed backprojection (scatter
forward projector) and the transposed filter.  Checks: dot-product tests for
B and for A (to 1e-5), A^T against the FP64 oracle gradient, finite
differences of ||A p - t||^2 at 32 pixels, and 20 steps of gradient descent.
"""
import numpy as np
import pytest

from _util import rel_rmse, small_geometry
from tomokvas_gb300 import _lib, device
from tomokvas_gb300.phantom import head_phantom

pytestmark = pytest.mark.gpu

DOT_TOL = 1e-5


def dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


# Row steps of consecutive slices, |scale| D / (D + W/2), below, near and
# above one detector row: "fine_voxels" (0.36: several slices share a row, the
# most shared-atomic collisions), "half_row" (0.60), "plain" (0.95) and
# "flips_scale" (1.43).  They also cover the three forms of the fixed-point box
# (at most 2^cbits contributions per cell): cbits 10 (both words with their
# bias subtraction), 9 (the hi word windowed) and 8, 7 (both words windowed).
GEOMS = {
    "plain": dict(W=64, N=72, H=56, vol=(48, 48, 40)),
    "flips_scale": dict(W=60, N=50, H=64, vol=(40, 36, 45), voxel_mm=1.2, dirx=1, dirz=1, rot=0.4),
    "fine_voxels": dict(W=64, N=40, H=48, vol=(48, 40, 36), voxel_mm=0.3),
    "half_row": dict(W=64, N=48, H=56, vol=(40, 44, 38), voxel_mm=0.5, diry=1, rot=0.2),
}


@pytest.mark.parametrize("fp_variant", [0, 2])
@pytest.mark.parametrize("name", list(GEOMS))
def test_forward_project_is_transpose_of_backproject(cuda, name, fp_variant):
    """<B q, y> = <q, B^T y> for the FP32-atomic and the fixed-point scatter."""
    import torch

    L = _lib.load()
    _lib.check(L.tk_fp_select_variant(fp_variant))
    try:
        _transpose_check(name, torch)
    finally:
        _lib.check(L.tk_fp_select_variant(0))


def _transpose_check(name, torch):
    g = small_geometry(**GEOMS[name])
    rng = np.random.default_rng(1)
    q = np.zeros((g.N, g.H, device.row_pitch(g.W)), dtype=np.float32)
    q[:, :, :g.W] = rng.normal(size=(g.N, g.H, g.W))
    y = rng.normal(size=(g.Z, g.Y, g.X)).astype(np.float32)
    Bq = device.backproject(g, dev(q, torch), None).cpu().numpy()
    Bty = device.forward_project(g, dev(y, torch)).cpu().numpy()
    lhs = float(np.sum(Bq.astype(np.float64) * y))
    rhs = float(np.sum(q[:, :, :g.W].astype(np.float64) * Bty[:, :, :g.W]))
    assert abs(lhs - rhs) <= DOT_TOL * abs(lhs)
    assert device.device_error_flags() == 0


@pytest.mark.parametrize("name", list(GEOMS))
def test_forward_projector_forms_agree(cuda, name):
    """Slice lanes (default), column lanes and the fixed-point slice-lane box
    scatter the same weights: the projections agree to FP32 rounding of the
    summation order, including a partial z chunk (Z not a multiple of 32)."""
    import torch

    L = _lib.load()
    g = small_geometry(**GEOMS[name])
    y = np.random.default_rng(4).normal(size=(g.Z, g.Y, g.X)).astype(np.float32)
    out = []
    try:
        for v in (0, 1, 2):
            _lib.check(L.tk_fp_select_variant(v))
            out.append(device.forward_project(g, dev(y, torch)).cpu().numpy()[:, :, :g.W])
    finally:
        _lib.check(L.tk_fp_select_variant(0))
    assert rel_rmse(out[0], out[1]) < 1e-6
    assert rel_rmse(out[2], out[0]) < 1e-6
    assert device.device_error_flags() == 0


@pytest.mark.parametrize("window", ["ramlak", "hann"])
@pytest.mark.parametrize("layout", ["sinogram", "projection"])
def test_fdk_dot_product(cuda, window, layout):
    import torch

    g = small_geometry(**GEOMS["plain"])
    rng = np.random.default_rng(2)
    shape = (g.H, g.N, g.W) if layout == "sinogram" else (g.N, g.H, g.W)
    x = rng.normal(size=shape).astype(np.float32)
    y = rng.normal(size=(g.Z, g.Y, g.X)).astype(np.float32)
    w, lay = _lib.WINDOWS[window], _lib.LAYOUTS[layout]
    Ax = device.fdk_device(g, dev(x, torch), _lib.TK_INPUT_F32, lay, window=w).cpu().numpy()
    Aty = device.fdk_backward(g, dev(y, torch), w, lay).cpu().numpy()
    lhs = float(np.sum(Ax.astype(np.float64) * y))
    rhs = float(np.sum(x.astype(np.float64) * Aty))
    assert abs(lhs - rhs) <= DOT_TOL * abs(lhs)


@pytest.mark.parametrize("name", list(GEOMS))
def test_backward_matches_fp64_gradient(orc, cuda, name):
    import torch

    g = small_geometry(**GEOMS[name])
    G = orc.geom_from(g)
    rng = np.random.default_rng(3)
    y = rng.normal(size=(g.Z, g.Y, g.X)).astype(np.float32)
    got = device.fdk_backward(g, dev(y, torch)).cpu().numpy()
    ref = orc.fdk_adjoint_f64(y, G)
    assert rel_rmse(got, ref) < 1e-5


def test_finite_differences_of_volume_loss(orc, cuda):
    """d/dp_i ||A p - t||^2 at 32 random detector samples, central differences."""
    import torch

    g = small_geometry(**GEOMS["plain"])
    G = orc.geom_from(g)
    ell = head_phantom(g.fov_radius_cm * 0.8, seed=6)
    p = orc.project_ellipsoids(ell, G, "sino")
    t = orc.voxelise_ellipsoids(ell, G)
    p_d = dev(p, torch)

    def loss(pp):
        v = device.fdk_device(g, pp).double()
        return float(torch.sum((v - dev(t, torch).double()) ** 2).item())

    r = device.fdk_device(g, p_d) - dev(t, torch)
    grad = (2.0 * device.fdk_backward(g, r)).cpu().numpy()
    rng = np.random.default_rng(4)
    idx = [tuple(rng.integers(0, n) for n in p.shape) for _ in range(32)]
    eps = 0.5  # the loss is exactly quadratic, so a large step has no truncation error
    errs = []
    for i in idx:
        pp = p_d.clone()
        pp[i] += eps
        lp = loss(pp)
        pp[i] -= 2 * eps
        lm = loss(pp)
        fd = (lp - lm) / (2 * eps)
        errs.append(abs(fd - grad[i]) / (abs(grad[i]) + 1e-3 * np.abs(grad).max()))
    assert max(errs) < 1e-3


def test_gradient_descent_data_consistency(orc, cuda):
    """20 steps of p <- p - a grad ||A p - t||^2 lower the loss monotonically."""
    import torch

    g = small_geometry(**GEOMS["plain"])
    G = orc.geom_from(g)
    ell = head_phantom(g.fov_radius_cm * 0.8, seed=7)
    rng = np.random.default_rng(5)
    p = orc.project_ellipsoids(ell, G, "sino")
    noisy = p + rng.normal(scale=0.01 * p.max(), size=p.shape).astype(np.float32)
    t = dev(orc.voxelise_ellipsoids(ell, G), torch)
    pk = dev(noisy, torch)
    # step from a power-iteration estimate of ||A||^2
    v = torch.randn_like(pk)
    for _ in range(8):
        v = device.fdk_backward(g, device.fdk_device(g, v))
        nrm = torch.linalg.vector_norm(v)
        v = v / nrm
    step = 0.9 / float(nrm.item())
    losses = []
    for _ in range(20):
        r = device.fdk_device(g, pk) - t
        losses.append(float(torch.sum(r.double() ** 2).item()))
        pk = pk - step * device.fdk_backward(g, r)
    assert all(b < a for a, b in zip(losses, losses[1:]))
    assert losses[-1] < 0.9 * losses[0]
