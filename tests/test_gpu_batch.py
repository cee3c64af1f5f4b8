"""Batches of uneven reconstructions (tk_batch_*): one persistent
backprojection launch over every item's voxel tiles, eager or as a replayed
CUDA graph.

Checks:
  * every item equals tk_fdk_device on the same input bit for bit, for each
    storage format's default tile shape (the arithmetic and its order are the
    per-volume kernel's; an item with the quarter-turn symmetry gets the
    per-volume quarter-turn launch); items cover sinogram and projection layouts, FP32
    line integrals and raw uint16 counts, Ram-Lak and Hann, axis flips and a
    rotation offset, scale != 1, a volume thinner than one z chunk and one
    whose depth is not a multiple of it;
  * a graph replay equals the eager run, and replays read the inputs anew;
  * after the autotuner picks each item's filter form (FFT or tensor-core
    Toeplitz product, by timing) and a tile shape, every item stays within
    the FP16 bound (5e-4 relative RMSE) of the FP64 oracle.
"""
import numpy as np
import pytest

from _util import rel_rmse, small_geometry
from tomokvas_gb300 import _lib, device
from tomokvas_gb300.batch import Batch, variants
from tomokvas_gb300.phantom import counts_u16, head_phantom

pytestmark = pytest.mark.gpu

ITEMS = [
    dict(geo=dict(W=64, N=72, H=56, vol=(48, 48, 40)), layout="sinogram", window="ramlak", raw=False),
    dict(geo=dict(W=48, N=50, H=48, vol=(32, 36, 30), dirx=1, rot=0.3), layout="sinogram", window="ramlak",
         raw=False),
    dict(geo=dict(W=64, N=90, H=64, vol=(40, 40, 100)), layout="projection", window="hann", raw=False),
    dict(geo=dict(W=32, N=40, H=32, vol=(24, 24, 24)), layout="projection", window="hann", raw=True),
    dict(geo=dict(W=96, N=60, H=80, vol=(64, 64, 70), voxel_mm=1.0, diry=1, dirz=1), layout="sinogram",
         window="shepp_logan", raw=False),
    # quarter-turn symmetry (square centred volume of whole 32-column tile pairs, N divisible by 4):
    # backprojected by tk_fdk_device's quarter-turn launch inside the batch run
    dict(geo=dict(W=64, N=80, H=56, vol=(64, 64, 40)), layout="projection", window="hann", raw=False),
]
QUAD = [False] * 5 + [True]
I0 = 60000.0


@pytest.fixture(scope="module")
def items(orc, cuda):
    import torch

    out = []
    for k, it in enumerate(ITEMS):
        g = small_geometry(**it["geo"])
        G = orc.geom_from(g)
        ell = head_phantom(g.fov_radius_cm * 0.85, seed=20 + k)
        lay = "sino" if it["layout"] == "sinogram" else "proj"
        p = orc.project_ellipsoids(ell, G, lay)
        if it["raw"]:
            host = counts_u16(p, I0, seed=30 + k)
            d_in = torch.from_numpy(host.view(np.int16)).cuda()
            ff = device.flatfield(flat_value=I0)
            itype = _lib.TK_INPUT_U16
        else:
            host, d_in, ff, itype = p, torch.from_numpy(p).cuda(), None, _lib.TK_INPUT_F32
        out.append(dict(g=g, G=G, host=host, d_in=d_in, ff=ff, itype=itype, layout=_lib.LAYOUTS[it["layout"]],
                        window=_lib.WINDOWS[it["window"]]))
    return out


def single(it, precision):
    return device.fdk_device(it["g"], it["d_in"], it["itype"], it["layout"], ff=it["ff"], window=it["window"],
                             precision=precision)


def make_batch(items, precision):
    import torch

    b = Batch(precision)
    vols = []
    for it in items:
        v = torch.full((it["g"].Z, it["g"].Y, it["g"].X), float("nan"), device="cuda")
        b.submit(it["g"], it["d_in"], v, it["itype"], it["layout"], it["ff"], it["window"])
        vols.append(v)
    b.plan()
    return b, vols


@pytest.mark.parametrize("precision", [_lib.TK_F16, _lib.TK_BF16, _lib.TK_F32_COEF])
def test_batch_equals_per_volume(items, precision):
    import torch

    b, vols = make_batch(items, precision)
    # the 16-bit formats take the quarter-turn launch where it applies; FP32 coefficients keep
    # their general walk (their quarter-turn variant is selectable only), as tk_fdk_device does
    assert b.quarter_turn_items() == (QUAD if precision != _lib.TK_F32_COEF else [False] * len(QUAD))
    b.run(graph=False)
    torch.cuda.synchronize()
    for it, v in zip(items, vols):
        np.testing.assert_array_equal(v.cpu().numpy(), single(it, precision).cpu().numpy())
    assert device.device_error_flags() == 0
    b.close()


def test_batch_many_units_per_cta(cuda):
    """Three 192^2 x 130 volumes: two for the persistent kernel (432 units each
    at the default tile shape, the last z chunk of each tile column ragged:
    several units per persistent CTA, so every CTA's mbarrier ring runs on
    across units of different items) and one with the quarter-turn symmetry
    (N = 84, unflipped in x and y) beside it.  Bit for bit against
    tk_fdk_device."""
    import torch

    geos = [small_geometry(W=256, N=90, H=200, vol=(192, 192, 130), voxel_mm=1.0),
            small_geometry(W=256, N=96, H=200, vol=(192, 192, 130), voxel_mm=1.1, dirx=1, rot=0.2),
            small_geometry(W=240, N=84, H=180, vol=(192, 192, 130), voxel_mm=0.9, dirz=1)]
    b = Batch(_lib.TK_F16)
    ins, vols = [], []
    for k, g in enumerate(geos):
        ins.append(device.phantom_project(g, head_phantom(g.fov_radius_cm * 0.85, seed=40 + k),
                                          _lib.TK_LAYOUT_SINOGRAM))
        vols.append(torch.full((g.Z, g.Y, g.X), float("nan"), device="cuda"))
        b.submit(g, ins[-1], vols[-1], _lib.TK_INPUT_F32, _lib.TK_LAYOUT_SINOGRAM, None, _lib.TK_WINDOW_HANN)
    b.plan()
    assert b.quarter_turn_items() == [False, False, True]
    b.run(graph=False)
    torch.cuda.synchronize()
    for g, x, v in zip(geos, ins, vols):
        ref = device.fdk_device(g, x, _lib.TK_INPUT_F32, _lib.TK_LAYOUT_SINOGRAM, window=_lib.TK_WINDOW_HANN,
                                precision=_lib.TK_F16)
        np.testing.assert_array_equal(v.cpu().numpy(), ref.cpu().numpy())
    assert device.device_error_flags() == 0
    b.close()


def test_graph_replay_equals_eager_and_rereads_inputs(items):
    import torch

    b, vols = make_batch(items, _lib.TK_F16)
    b.run(graph=False)
    torch.cuda.synchronize()
    eager = [v.cpu().numpy() for v in vols]
    for v in vols:
        v.fill_(float("nan"))
    b.run(graph=True)
    b.run(graph=True)
    torch.cuda.synchronize()
    for e, v in zip(eager, vols):
        np.testing.assert_array_equal(v.cpu().numpy(), e)
    # replays read the submitted inputs anew: doubling an FP32 input doubles its volume
    items[0]["d_in"].mul_(2.0)
    try:
        b.run(graph=True)
        torch.cuda.synchronize()
        np.testing.assert_allclose(vols[0].cpu().numpy(), 2.0 * eager[0], rtol=1e-6, atol=1e-6 * np.abs(eager[0]).max())
        np.testing.assert_array_equal(vols[1].cpu().numpy(), eager[1])
    finally:
        items[0]["d_in"].mul_(0.5)
    b.close()


def test_autotuned_batch_vs_fp64(orc, items):
    import torch

    b, vols = make_batch(items, _lib.TK_F16)
    name, ms = b.autotune()
    assert name in [n for _, n in variants(_lib.TK_F16)] and ms > 0
    assert b.variant == name
    # each item's filter form was chosen by timing: the FFT or (W <= 512) the tensor-core product
    forms = b.filter_forms()
    assert len(forms) == len(items)
    for it, f in zip(items, forms):
        assert f in (_lib.TK_FILTER_FFT, _lib.TK_FILTER_TOEPLITZ)
        assert f == _lib.TK_FILTER_FFT or it["g"].W <= 512
    for v in vols:
        v.fill_(float("nan"))
    b.run(graph=True)
    torch.cuda.synchronize()
    for it, v in zip(items, vols):
        if it["itype"] == _lib.TK_INPUT_U16:
            ref = orc.fdk_u16_f64_sampled(it["host"], it["G"], I0, window=it["window"],
                                          zlist=np.arange(it["g"].Z, dtype=np.int32))
        else:
            sino = it["host"] if it["layout"] == _lib.TK_LAYOUT_SINOGRAM else np.transpose(it["host"], (1, 0, 2))
            ref = orc.fdk_f64(np.ascontiguousarray(sino), it["G"], it["window"])
        assert rel_rmse(v.cpu().numpy(), ref) < 5e-4
    assert device.device_error_flags() == 0
    b.close()
