"""Pins the rsq steps against the reference itself: golden outputs of
Lukas-kV/TomoKvas's own FBPG/rsq_load.cpp (class rsq: LoadImages +
ProccessAndCopy, compiled from the reference's source on the CPU by
oracle/ref_build.py.build_rsq; tests/golden/make_rsq_golden.py) on a
synthetic .RSQ scan of two detector rows of the reference's fixed 1024 x 2000
sinogram.

CPU: the flat field + log formula (FlatFieldCorrection, rsq_load.cpp:299-325),
in double and through the oracle (FP32 output), and the oracle's FP64
restatements of Half2FullFan (:327-380) and Half2Para / Fan2Para (:382-470),
against the reference's rows.
GPU: the rebinning kernels (tk_half_to_full_fan, tk_half_to_parallel) and the
flat field fused into the filter's load (per-pixel dark and flat maps), against
the reference's outputs.

Bounds (relative to max |reference|): double formula 1e-13; oracle FP32 log
1e-6; FP64 restatements 1e-12; GPU kernels (FP32 samples) 2e-6; GPU filtered
rows of the raw counts vs of the reference's flat field: relative RMSE 1e-5.
"""
import glob
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_rsq_golden as mk  # noqa: E402

FIX = {os.path.basename(p)[4:-4]: p for p in glob.glob(os.path.join(HERE, "golden", "rsq_*.npz"))}


def fixture(name):
    return np.load(FIX[name])


def flat_field(invert=True):
    """The reference's formula in double: A log((I - dark) / (flat - dark)) + B, negated when inverted,
    over the regenerated counts; [rows][N][W]."""
    counts, dark, flat = mk.rsq_counts()
    bx, by = mk.BH_X, mk.BH_Y
    A = (by[2] - by[0]) / (bx[2] - bx[0])
    B = by[0] - A * bx[0]
    num = counts.astype(np.int64) - dark[:, None, :].astype(np.int64)
    den = (flat.astype(np.int64) - dark.astype(np.int64))[:, None, :].astype(np.float64)
    v = A * np.log(num / den) + B
    return -v if invert else v


def test_rsq_fixtures_present():
    assert set(FIX) >= set(mk.CASES)


@pytest.mark.parametrize("name,invert", [("ff", True), ("ff_plain", False)])
def test_flat_field_matches_reference(orc, name, invert):
    d = fixture(name)
    ref = d["out"]
    rows = d["rows"]
    ff = flat_field(invert)
    assert tuple(d["shape"]) == ff.shape
    scale = np.abs(ref).max()
    assert np.abs(ff[:, rows, :] - ref).max() <= 1e-13 * scale
    counts, dark, flat = mk.rsq_counts()
    bx, by = mk.BH_X, mk.BH_Y
    A = (by[2] - by[0]) / (bx[2] - bx[0])
    sino = orc.log_u16(np.ascontiguousarray(np.transpose(counts, (1, 0, 2))), flat.astype(np.float32),
                       dark=dark.astype(np.float32), A=A, B=by[0] - A * bx[0], invert=invert)  # [rows][N][W]
    assert np.abs(sino[:, rows, :] - ref).max() <= 1e-6 * scale


@pytest.mark.parametrize("name", ["fullfan", "fullfan_flip", "para"])
def test_rebinning_restatements_match_reference(orc, name):
    d = fixture(name)
    am, comp, para, flip, inv = (int(x) for x in d["settings"])
    ff = flat_field(bool(inv))
    if para:
        out = orc.half2para(ff, am, float(d["distance"]), float(d["dfi"]))
    else:
        out = orc.half2fullfan(ff, am, float(d["distance"]), float(d["dfi"]), bool(flip))
    assert out.shape == tuple(d["shape"])
    ref = d["out"]
    assert np.abs(out[:, d["rows"], :] - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["fullfan", "fullfan_flip", "para"])
def test_gpu_rebinning_matches_reference(cuda, name):
    import torch

    from tomokvas_gb300 import device

    d = fixture(name)
    am, comp, para, flip, inv = (int(x) for x in d["settings"])
    x = torch.from_numpy(flat_field(bool(inv)).astype(np.float32)).cuda()
    if para:
        out = device.half_to_parallel(x, am, float(d["distance"]), float(d["dfi"]))
    else:
        out = device.half_to_full_fan(x, am, float(d["distance"]), float(d["dfi"]), bool(flip))
    got = out.cpu().numpy()
    assert got.shape == tuple(d["shape"])
    ref = d["out"]
    assert np.abs(got[:, d["rows"], :] - ref).max() <= 2e-6 * np.abs(ref).max()


@pytest.mark.gpu
def test_gpu_fused_flat_field_matches_reference(cuda):
    """The filter's fused load of raw counts with per-pixel dark and flat rows gives the same
    filtered rows as the filter of the reference's flat-field output."""
    import torch

    from _util import rel_rmse
    from tomokvas_gb300 import _lib, device
    from tomokvas_gb300.geometry import FDKGeometry

    d = fixture("ff")
    counts, dark, flat = mk.rsq_counts()
    bx, by = mk.BH_X, mk.BH_Y
    A = (by[2] - by[0]) / (bx[2] - bx[0])
    g = FDKGeometry(W=mk.W, N=mk.N, H=mk.ROWS, cX=(mk.W - 1) / 2.0, cZ=0.5, dfi=float(d["dfi"]),
                    D=float(d["distance"]), tau=0.01, X=64, Y=64, Z=2, cx=31.5, cy=31.5)
    dk = torch.from_numpy(dark.astype(np.float32)).cuda()
    fl = torch.from_numpy(flat.astype(np.float32)).cuda()
    ff = device.flatfield(flat=fl, dark=dk, A=A, B=by[0] - A * bx[0], invert=True, floor_counts=0.5)
    raw = torch.from_numpy(counts.view(np.int16)).cuda()  # sinogram-major [rows][N][W]
    q_raw, _ = device.filter_projections(g, raw, _lib.TK_INPUT_U16, _lib.TK_LAYOUT_SINOGRAM, ff=ff)
    ref_ff = torch.from_numpy(flat_field(True).astype(np.float32)).cuda()  # the reference's output (all rows)
    assert np.abs(flat_field(True)[:, d["rows"], :] - d["out"]).max() <= 1e-13 * np.abs(d["out"]).max()
    q_ref, _ = device.filter_projections(g, ref_ff, _lib.TK_INPUT_F32, _lib.TK_LAYOUT_SINOGRAM)
    torch.cuda.synchronize()
    assert device.device_error_flags() == 0
    assert rel_rmse(q_raw.cpu().numpy(), q_ref.cpu().numpy()) < 1e-5
