"""Half-fan completion and fan->parallel rebinning oracle (rsq_load.cpp:327-470), no GPU.

The C oracle is checked against a line-by-line Python restatement of the
reference's loops on a small case, and against a closed form: for fan-beam
data of a disk centred on the rotation axis, every ray's value depends only
on its distance from the centre, so completion reproduces the data of a full
detector exactly and rebinning gives the parallel-beam profile.
"""
import math

import numpy as np

from oracle import oracle as orc


def py_half2fullfan(img, am, D, dfi, flip):
    N, W = img.shape
    Wc, c0 = 2 * W - 1 - 2 * am, W - 1 - am
    out = np.zeros((N, Wc))
    for f in range(N):
        row = out[N - 1 - f] if flip else out[f]
        row[c0:] = img[f, am:]
        fi = f * dfi
        for t in range(-c0, 0):
            at = math.atan(t / D)
            nf = (fi - 2 * at - math.pi) / dfi
            if nf > N - 1 or nf < 0:
                nf = (fi - 2 * at + math.pi) / dfi
            a, b = math.ceil(nf), math.floor(nf)
            A = img[a - N, -t + am] if a > N - 1 else img[a, -t + am]
            B = img[b, -t + am]
            row[t + c0] = A + (B - A) * (a - nf) if a != b else A
    return out


def py_half2para(img, am, D, dfi):
    N, W = img.shape
    Wc, center = 2 * W - 1 - 2 * am, W - 1 - am
    out = np.zeros((N // 2, Wc))
    for f in range(N // 2):
        for u in range(Wc):
            ui = u - center
            beta = f + math.asin(ui / D) / dfi if ui >= 0 else f - (math.asin(ui / D) - math.pi) / dfi
            if beta < 0:
                beta += N
            if beta > N - 1:
                beta -= N
            col = math.ceil(abs(ui)) + am
            ba, bb = math.ceil(beta), math.floor(beta)
            if ba != bb:
                va, vb = img[ba, col], img[bb if bb >= 0 else bb + N, col]
                out[f, u] = va + (vb - va) * (ba - beta)
            else:
                out[f, u] = img[ba, col]
    return out


def test_oracle_matches_python_restatement():
    rng = np.random.default_rng(0)
    N, W, am, D = 24, 10, 2, 40.0
    dfi = 2 * math.pi / N
    img = rng.normal(size=(2, N, W))
    for flip in (False, True):
        got = orc.half2fullfan(img, am, D, dfi, flip)
        for r in range(2):
            np.testing.assert_allclose(got[r], py_half2fullfan(img[r], am, D, dfi, flip), rtol=0, atol=1e-13)
    got = orc.half2para(img, am, D, dfi)
    for r in range(2):
        np.testing.assert_allclose(got[r], py_half2para(img[r], am, D, dfi), rtol=0, atol=1e-13)


def disk_fan(N, W, am, D, R):
    """Fan-beam chord lengths of a centred disk of radius R (pixels) on a flat detector whose column
    am holds the central ray; columns t = x - am (negative t are the unmeasured half)."""
    t = np.arange(-(W - 1 - am), W - am, dtype=np.float64)  # full detector offsets
    d = D * np.abs(t) / np.sqrt(D * D + t * t)  # distance of the ray from the centre
    chord = 2 * np.sqrt(np.maximum(R * R - d * d, 0.0))
    return np.tile(chord, (N, 1)), t


def test_completion_of_a_centred_disk_is_exact():
    N, W, am, D, R = 180, 64, 6, 400.0, 40.0
    full, t = disk_fan(N, W, am, D, R)  # [N][2W-1-2am]
    half = full[:, W - 1 - am - am:]  # the measured columns: offsets -am .. W-1-am
    assert half.shape == (N, W)
    got = orc.half2fullfan(half[None], am, D, 2 * math.pi / N)[0]
    np.testing.assert_allclose(got, full, rtol=0, atol=1e-12)


def test_parallel_rebinning_of_a_centred_disk():
    N, W, am, D, R = 360, 64, 6, 400.0, 40.0
    full, t = disk_fan(N, W, am, D, R)
    half = full[:, W - 1 - am - am:]
    par = orc.half2para(half[None], am, D, 2 * math.pi / N)[0]  # [N/2][Wc]
    # the rebinned column s samples the fan column |s| + am: chord of the ray at distance D|s|/sqrt(D^2+s^2)
    s = np.arange(par.shape[1]) - (W - 1 - am)
    d = D * np.abs(s) / np.sqrt(D * D + s * s)
    np.testing.assert_allclose(par, np.tile(2 * np.sqrt(np.maximum(R * R - d * d, 0)), (N // 2, 1)), atol=1e-12)
