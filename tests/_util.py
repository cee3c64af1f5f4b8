"""Shared helpers of the test-suite (error metrics, small workloads)."""
import numpy as np

from tomokvas_gb300.geometry import FDKGeometry


def rel_rmse(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-300))


def max_abs(a, b):
    return float(np.max(np.abs(np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64))))


def small_geometry(W=64, N=120, H=64, vol=(64, 64, 64), pitch_mm=1.6, voxel_mm=0.8, **kw):
    """A scaled-down version of the 180 x 256^2 workload (SOD 500, SDD 1000)."""
    return FDKGeometry.circular(N, W, H, pitch_mm, 500.0, 1000.0, vol, voxel_mm, **kw)
