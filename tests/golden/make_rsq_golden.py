"""Generates the rsq golden fixtures: outputs of the reference's own rsq reader.

Writes a synthetic Scanco .RSQ scan (two detector rows of the reference's
fixed 1024-column x 2000-projection sinogram, seeded uint16 counts, dark and
flat rows, a beam-hardening line) and runs Lukas-kV/TomoKvas FBPG/rsq_load.cpp
(compiled by oracle/ref_build.py.build_rsq, driven by oracle/tk_rsqrun.cpp)
through LoadImages + ProccessAndCopy in four settings:

  ff        flat field + log (FlatFieldCorrection, rsq_load.cpp:299-325),
            inverted, no completion (axis_move 0: CutHalfSin copies it whole)
  ff_plain  the same without inversion
  fullfan   Half2FullFan completion (rsq_load.cpp:327-380), axis_move 21
  fullfan_flip   the same, flipped
  para      Half2Para / Fan2Para rebinning (rsq_load.cpp:382-470)

Each fixture stores the settings, the seed of the counts (regenerated by
rsq_counts below at test time), and every 125th output row of each sinogram
in float64.  CPU only:

    python tests/golden/make_rsq_golden.py [out_dir]
"""
import ctypes
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_build  # noqa: E402
from tomokvas_gb300.scanfile import write_rsq  # noqa: E402

W, N, ROWS = 1024, 2000, 2          # the reference's fixed sinogram size (rsq_load.cpp:13-15)
DISTANCE = 125810.0 / 24.0          # its default source distance in pixels (rsq_load.cpp:23)
DFI = 2.0 * np.pi / N
BH_X, BH_Y = (120, 260, 410), (0.85, 1.9, 3.2)
SEED = 2024
ROW_STEP = 125

CASES = {  # name: (axis_move, complete, parallel, flip, invert)
    "ff": (0, 0, 0, 0, 1),
    "ff_plain": (0, 0, 0, 0, 0),
    "fullfan": (21, 1, 0, 0, 1),
    "fullfan_flip": (21, 1, 0, 1, 1),
    "para": (21, 1, 1, 0, 1),
}


def rsq_counts(seed=SEED):
    """Counts [ROWS][N][W], dark and flat rows [ROWS][W] of the synthetic scan: a smooth attenuation
    profile (a shifted disc per angle, so half-fan completion has structure to interpolate) with
    Poisson noise."""
    rng = np.random.default_rng(seed)
    x = np.arange(W) - 300.0
    b = np.arange(N)[:, None]
    prof = 1.2 * np.sqrt(np.clip(1.0 - ((x[None, :] - 80.0 * np.sin(2 * np.pi * b / N)) / 420.0) ** 2, 0, 1))
    dark = rng.integers(20, 60, size=(ROWS, W)).astype(np.uint16)
    flat = rng.integers(52000, 60000, size=(ROWS, W)).astype(np.uint16)
    counts = np.empty((ROWS, N, W), dtype=np.uint16)
    for r in range(ROWS):
        lam = dark[r].astype(np.float64) + (flat[r] - dark[r]) * np.exp(-(0.8 + 0.2 * r) * prof)
        counts[r] = np.clip(rng.poisson(lam), 61, 65535).astype(np.uint16)
    return counts, dark, flat


def run_reference(path, axis_move, complete, parallel, flip, invert):
    L = ctypes.CDLL(ref_build.build_rsq())
    u = ctypes.c_uint
    L.tkref_rsq.argtypes = [ctypes.c_char_p, u, u, u, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                            ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(u), ctypes.POINTER(u)]
    w, h = u(0), u(0)
    args = [path.encode(), 0, ROWS - 1, axis_move, DISTANCE, DFI, complete, parallel, flip, invert]
    assert L.tkref_rsq(*args, None, ctypes.byref(w), ctypes.byref(h)) == 0
    out = np.zeros((ROWS, h.value, w.value), dtype=np.float64)
    assert L.tkref_rsq(*args, out.ctypes.data, None, None) == 0
    return out


def main(out_dir):
    counts, dark, flat = rsq_counts()
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "scan.rsq")
        write_rsq(path, counts, dark, flat, bh_x=BH_X, bh_y=BH_Y)
        for name, (am, comp, para, flip, inv) in CASES.items():
            out = run_reference(path, am, comp, para, flip, inv)
            rows = np.arange(0, out.shape[1], ROW_STEP)
            np.savez_compressed(os.path.join(out_dir, f"rsq_{name}.npz"), rows=rows.astype(np.int32),
                                out=out[:, rows, :], shape=np.array(out.shape), seed=np.int64(SEED),
                                settings=np.array([am, comp, para, flip, inv]),
                                distance=np.float64(DISTANCE), dfi=np.float64(DFI),
                                bh=np.array(BH_X + BH_Y, dtype=np.float64))
            print(name, out.shape, float(np.abs(out).max()))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
