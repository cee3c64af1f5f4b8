"""Half-fan completion and fan->parallel rebinning on the GPU (tk_half_to_full_fan,
tk_half_to_parallel) against the FP64 restatement of rsq_load.cpp:327-470: the
kernels index in FP64 like the reference and store FP32, so the bound is FP32
rounding of the samples (max error <= 1e-6 of the data range)."""
import math

import numpy as np
import pytest

from tomokvas_gb300 import device

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,N,am,D,flip", [(40, 90, 5, 300.0, False), (33, 120, 0, 150.5, True), (64, 360, 12, 900.0, False)])
def test_half_fan_completion_and_rebinning(orc, cuda, W, N, am, D, flip):
    import torch

    rng = np.random.default_rng(W + N)
    sino = rng.normal(size=(3, N, W)).astype(np.float32)
    dfi = 2 * math.pi / N
    d = torch.from_numpy(sino).cuda()
    full = device.half_to_full_fan(d, am, D, dfi, flip).cpu().numpy()
    ref = orc.half2fullfan(sino.astype(np.float64), am, D, dfi, flip)
    rng_ = np.abs(sino).max()
    assert full.shape == ref.shape and np.abs(full - ref).max() <= 1e-6 * rng_
    par = device.half_to_parallel(d, am, D, dfi).cpu().numpy()
    refp = orc.half2para(sino.astype(np.float64), am, D, dfi)
    assert par.shape == refp.shape and np.abs(par - refp).max() <= 1e-6 * rng_
