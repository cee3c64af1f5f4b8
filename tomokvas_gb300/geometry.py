"""Reference parameter set of the FDK hot path and the named workloads.

The fields are exactly those the reference engine receives
(Lukas-kV/TomoKvas FBPG/kernel.cu:479-537 and FBPG/para_TC.cpp:130-142):
a flat virtual detector through the rotation axis with pitch ``tau`` (cm),
source distance ``D`` in virtual pixels, volume voxel pitch ``scale`` in
virtual pixels.  ``circular`` maps a physical circular cone-beam scan onto
them: tau_iso = pitch*SOD/SDD, D = SOD/tau_iso = SDD/pitch, scale = voxel/tau_iso.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, replace

import numpy as np

from ._lib import Geometry


@dataclass
class FDKGeometry:
    W: int
    N: int
    H: int
    cX: float
    cZ: float
    dfi: float
    D: float
    tau: float
    X: int
    Y: int
    Z: int
    cx: float
    cy: float
    cz: float = 0.0
    rot: float = 0.0
    scale: float = 1.0
    dirx: int = 0
    diry: int = 0
    dirz: int = 0
    zb: int = 16  # slices per Z block of the reference schedule (SetBlockSize)

    @classmethod
    def circular(cls, n_proj, det_cols, det_rows, pitch_mm, sod_mm, sdd_mm, vol, voxel_mm, **kw):
        tau_mm = pitch_mm * sod_mm / sdd_mm
        X, Y, Z = vol
        # delta_fi = 2*PI/N in double, handed over as float (mucat_file.cpp:141, para_TC.cpp:82)
        dfi = float(np.float32(2.0 * math.pi / n_proj))
        g = cls(W=det_cols, N=n_proj, H=det_rows, cX=(det_cols - 1) / 2.0, cZ=(det_rows - 1) / 2.0,
                dfi=dfi, D=sod_mm / tau_mm, tau=tau_mm / 10.0, X=X, Y=Y, Z=Z,
                cx=(X - 1) / 2.0, cy=(Y - 1) / 2.0, cz=0.0, scale=voxel_mm / tau_mm)
        return replace(g, **kw) if kw else g

    def to_c(self) -> Geometry:
        g = Geometry()
        for name, _ in Geometry._fields_:
            setattr(g, name, getattr(self, name))
        return g

    def replace(self, **kw) -> "FDKGeometry":
        return replace(self, **kw)

    @property
    def updates(self) -> int:
        """Voxel-projection updates of one full reconstruction."""
        return self.X * self.Y * self.Z * self.N

    @property
    def fov_radius_cm(self) -> float:
        return self.W / 2.0 * self.tau

    @property
    def voxel_cm(self) -> float:
        return abs(self.scale) * self.tau


def config(name: str) -> FDKGeometry:
    """Geometries of the reference workloads (sizes as the benchmark names them)."""
    if name == "c1":  # 180 x 256^2 at 0.4 mm, SOD 500, SDD 1000 -> 256^3 at 0.2 mm
        return FDKGeometry.circular(180, 256, 256, 0.4, 500.0, 1000.0, (256, 256, 256), 0.2)
    if name == "c2":  # 720 x 1024^2 at 0.15 mm, SOD 300, SDD 900 -> 1024^3 (s = 1)
        return FDKGeometry.circular(720, 1024, 1024, 0.15, 300.0, 900.0, (1024, 1024, 1024), 0.05)
    if name == "c4":  # 360 x 768^2 -> 512^3 at s = 1.5
        return FDKGeometry.circular(360, 768, 768, 0.2, 400.0, 800.0, (512, 512, 512), 0.15)
    if name == "c5":  # 1440 x 2048^2 at 0.1 mm, SOD 400, SDD 1200 -> 2048^3 (s = 1)
        return FDKGeometry.circular(1440, 2048, 2048, 0.1, 400.0, 1200.0, (2048, 2048, 2048), 0.1 / 3.0)
    raise KeyError(name)
