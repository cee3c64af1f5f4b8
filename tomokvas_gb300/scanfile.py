"""Python side of the reference's scan and volume files (the C++ side is include/tk_io.hpp).

write_cra: a .CRA scan description plus its raw float32 projection file, in
the layout cra_con reads (FBPG/mucat_file.cpp:8-277): "KEY: value" lines, the
raw file holding num_of_blocks scan blocks of num_of_projections frames of
detector_z x detector_x float32, clockwise scans stored in decreasing angle
order.  read_binsiz: the volume a bin_siz-style writer produced
(FBPG/mucat_file.cpp:430-520): "X Y Z 0" in .siz, float32 [Z][Y][X] in .bin.
cra_geometry: the engine parameters the reference's driver derives from a
.CRA header (FBPG/para_TC.cpp:48-142 with cra_con's float arithmetic).
"""
from __future__ import annotations

import math
import os

import numpy as np

from .geometry import FDKGeometry


def write_cra(directory: str, name: str, projections, sample_spacing_um: float, distance_cm: float,
              centres, rotate_angle_deg: float = 0.0, clockwise: bool = False, x_dimension: int = 0,
              z_dimension: int = 0, scale: float = 1.0, source_name: str = "synthetic", crlf: bool = False) -> str:
    """projections: [blocks][N][H][W] (or [N][H][W]) float32 in increasing angle order."""
    p = np.asarray(projections, dtype=np.float32)
    if p.ndim == 3:
        p = p[None]
    blocks, N, H, W = p.shape
    centres = list(np.atleast_1d(centres))
    assert len(centres) == blocks
    raw = name + ".raw"
    with open(os.path.join(directory, raw), "wb") as f:
        for b in range(blocks):
            frames = p[b, ::-1] if clockwise else p[b]
            f.write(np.ascontiguousarray(frames).tobytes())
    lines = [f"FILE NAME:              {raw}", f"SOURCE NAME:            {source_name}",
             f"SAMPLE SPACING:         {sample_spacing_um!r}", f"DISTANCE:               {distance_cm!r}",
             f"DETECTOR X PIXELS:      {W}", f"DETECTOR Z PIXELS:      {H}",
             f"NUMBER OF PROJECTIONS:  {N}", f"X DIMENSION:            {x_dimension}",
             f"Z DIMENSION:            {z_dimension}", f"ROTATE ANGLE:           {rotate_angle_deg!r}",
             f"NUMBER OF BLOCKS:       {blocks}", f"SCALE:                  {scale!r}"]
    lines += [f"CENTRE:                 {float(c)!r}" for c in centres]
    if clockwise:
        lines.append("CLOCKWISE:")
    with open(os.path.join(directory, name + ".CRA"), "w", newline="") as f:
        f.write(("\r\n" if crlf else "\n").join(lines) + ("\r\n" if crlf else "\n"))
    return os.path.join(directory, name + ".CRA")


def read_binsiz(directory: str, name: str) -> np.ndarray:
    with open(os.path.join(directory, name + ".siz")) as f:
        x, y, z, _ = (int(t) for t in f.read().split())
    vol = np.fromfile(os.path.join(directory, name + ".bin"), dtype=np.float32)
    assert vol.size == x * y * z, (vol.size, x, y, z)
    return vol.reshape(z, y, x)


def cra_derived(sample_spacing_um, distance_cm, detector_x, detector_z, n_proj, x_dimension=0, z_dimension=0):
    """cra_con::GetMetaData's derived values with its float/int arithmetic
    (FBPG/mucat_file.cpp:139-161): (distance px, delta_fi, x_dimension, z_dimension)."""
    f32 = np.float32
    distance = f32(distance_cm * 10000.0 / sample_spacing_um)
    dfi = f32(2 * math.pi / n_proj)
    phi = np.arctan(f32(detector_x // 2) / distance, dtype=np.float32)
    tmp = 2 * int(f32(distance * np.sin(phi, dtype=np.float32)) + f32(1))
    if x_dimension > tmp or x_dimension < 1:
        x_dimension = tmp
    tmp = int(f32(f32(distance - f32(x_dimension // 2)) / distance) * f32(detector_z)) & ~1
    if z_dimension > tmp:
        z_dimension = tmp
    if z_dimension < 1:
        z_dimension = 1
    return float(distance), float(dfi), x_dimension, z_dimension


def cra_geometry(sample_spacing_um, distance_cm, detector_x, detector_z, n_proj, centre, rotate_angle_deg=0.0,
                 clockwise=False, x_dimension=0, z_dimension=0, scale=1.0, vertical_offset=0.0, zb=16,
                 dirs=(0, 0, 0)) -> FDKGeometry:
    """The parameters FBPG/para_TC.cpp hands the engine for one scan block (one angle block)."""
    distance, dfi, xd, zd = cra_derived(sample_spacing_um, distance_cm, detector_x, detector_z, n_proj,
                                        x_dimension, z_dimension)
    rec = xd if xd else detector_x
    rx = int(rec * scale)
    rz = int(zd * scale)
    rot = (float(np.float32(dfi)) if clockwise else 0.0) + rotate_angle_deg * math.pi / 180.0
    return FDKGeometry(W=detector_x, N=n_proj, H=detector_z, cX=float(np.float32(centre)),
                       cZ=(detector_z - 1) / 2.0 + vertical_offset, dfi=dfi, D=distance,
                       tau=float(np.float32(sample_spacing_um)) * 0.0001, X=rx, Y=rx, Z=rz,
                       cx=(rx - 1) / 2.0, cy=(rx - 1) / 2.0, cz=0.0, rot=float(np.float32(rot)),
                       scale=1.0 / scale, dirx=dirs[0], diry=dirs[1], dirz=dirs[2], zb=zb)
