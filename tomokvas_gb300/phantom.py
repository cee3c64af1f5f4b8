"""Seeded synthetic phantoms (sets of ellipsoids) and raw-count simulation.

Record format (16 doubles per ellipsoid, shared with the C ABI's
tk_phantom_project): centre[3] (cm), semi-axes[3] (cm), rotation
world->local[9] (row major), density (1/cm).  Densities of overlapping
ellipsoids add.  Coordinates are the volume frame of the backprojector.
"""
from __future__ import annotations

import numpy as np


def _rot_zx(phi: float, theta: float) -> np.ndarray:
    """World->local rotation: about z by phi, then about x by theta."""
    cz, sz = np.cos(phi), np.sin(phi)
    cx, sx = np.cos(theta), np.sin(theta)
    Rz = np.array([[cz, sz, 0.0], [-sz, cz, 0.0], [0.0, 0.0, 1.0]])
    Rx = np.array([[1.0, 0.0, 0.0], [0.0, cx, sx], [0.0, -sx, cx]])
    return Rx @ Rz


def ellipsoid(centre, axes, rho, phi=0.0, theta=0.0, R=None) -> np.ndarray:
    rec = np.zeros(16)
    rec[0:3] = centre
    rec[3:6] = axes
    rec[6:15] = (R if R is not None else _rot_zx(phi, theta)).reshape(9)
    rec[15] = rho
    return rec


# A head-like arrangement of 10 nested ellipsoids (relative units of the
# phantom radius): outer shell, interior, two cavities and small inserts.
_HEAD = [
    # centre (x, y, z)     semi-axes (x, y, z)    rho    phi(deg)
    ((0.00, 0.00, 0.00), (0.72, 0.88, 0.84), 1.00, 0.0),
    ((0.00, -0.02, 0.00), (0.68, 0.83, 0.80), -0.75, 0.0),
    ((0.25, 0.05, -0.10), (0.14, 0.30, 0.22), -0.15, 15.0),
    ((-0.24, 0.08, -0.05), (0.18, 0.36, 0.25), -0.15, -20.0),
    ((0.00, 0.40, 0.25), (0.22, 0.20, 0.18), 0.12, 0.0),
    ((0.00, 0.12, 0.00), (0.05, 0.05, 0.05), 0.10, 0.0),
    ((0.00, -0.12, 0.00), (0.05, 0.05, 0.05), 0.10, 0.0),
    ((-0.09, -0.55, -0.20), (0.05, 0.03, 0.06), 0.10, 30.0),
    ((0.07, -0.55, -0.20), (0.03, 0.03, 0.05), 0.10, 0.0),
    ((0.05, -0.20, 0.50), (0.07, 0.08, 0.12), 0.20, 0.0),
]


def head_phantom(radius_cm: float, seed: int = 0, jitter: float = 0.05, mu: float = 0.5) -> np.ndarray:
    """10-ellipsoid head-like phantom; centres, axes and densities jittered by +-jitter."""
    rng = np.random.default_rng(seed)
    recs = []
    for c, a, rho, phi in _HEAD:
        cj = np.array(c) + rng.uniform(-jitter, jitter, 3) * np.array(a)
        aj = np.array(a) * (1.0 + rng.uniform(-jitter, jitter, 3))
        rj = rho * (1.0 + rng.uniform(-jitter, jitter))
        recs.append(ellipsoid(cj * radius_cm, aj * radius_cm, rj * mu, phi=np.deg2rad(phi)))
    return np.stack(recs)


def random_ellipsoids(n: int, radius_cm: float, half_height_cm: float, seed: int = 0,
                      mu_range=(0.1, 2.0), axis_range=(0.05, 0.3)) -> np.ndarray:
    """n ellipsoids with random centres inside a cylinder, random axes and orientation."""
    rng = np.random.default_rng(seed)
    recs = []
    for _ in range(n):
        r = radius_cm * 0.55 * np.sqrt(rng.uniform())
        t = rng.uniform(0, 2 * np.pi)
        c = np.array([r * np.cos(t), r * np.sin(t), rng.uniform(-0.55, 0.55) * half_height_cm])
        a = rng.uniform(*axis_range, 3) * radius_cm
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        recs.append(ellipsoid(c, a, rng.uniform(*mu_range), R=q))
    return np.stack(recs)


def counts_u16(line_integrals: np.ndarray, I0: float, seed: int = 0) -> np.ndarray:
    """Poisson(I0 * exp(-p)) clipped to uint16."""
    rng = np.random.default_rng(seed)
    lam = I0 * np.exp(-np.asarray(line_integrals, dtype=np.float64))
    return np.clip(rng.poisson(lam), 0, 65535).astype(np.uint16)
