"""Python side of the reference's scan and volume files (the C++ side is include/tk_io.hpp).

write_cra: a .CRA scan description plus its raw float32 projection file, in
the layout cra_con reads (FBPG/mucat_file.cpp:8-277): "KEY: value" lines, the
raw file holding num_of_blocks scan blocks of num_of_projections frames of
detector_z x detector_x float32, clockwise scans stored in decreasing angle
order.  read_binsiz: the volume a bin_siz-style writer produced
(FBPG/mucat_file.cpp:430-520): "X Y Z 0" in .siz, float32 [Z][Y][X] in .bin.
cra_geometry: the engine parameters the reference's driver derives from a
.CRA header (FBPG/para_TC.cpp:48-142 with cra_con's float arithmetic).
write_rsq: a Scanco-style .RSQ raw scan in the layout rsq reads
(FBPG/rsq_load.h:13-59, FBPG/rsq_load.cpp:185-227, 488-548): the 512-byte
header block, the beam-hardening text at byte 3432, and from byte 3584 one
block per detector row (dark row, flat row, the row's projections) of uint16.
"""
from __future__ import annotations

import math
import os

import numpy as np

import struct

from .geometry import FDKGeometry

RSQ_DATA_OFFSET = 3584  # rsq_load.cpp:12
RSQ_BH_OFFSET = 3432    # rsq_load.cpp:506


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


def write_rsq(path: str, counts, dark, flat, bh_x=(100, 200, 300), bh_y=(1.0, 2.0, 3.0), name: str = "synthetic",
              header: dict | None = None) -> None:
    """counts: [rows][N][W] uint16 (each detector row's projections); dark, flat:
    [rows][W] uint16.  bh_x, bh_y: the three beam-hardening correction points.
    header: ima_data_type fields by name (rsq_load.h:13-48); the others are 0."""
    counts = np.ascontiguousarray(counts, dtype="<u2")
    dark = np.ascontiguousarray(dark, dtype="<u2")
    flat = np.ascontiguousarray(flat, dtype="<u2")
    rows, n, w = counts.shape
    fields = dict(nr_of_samples=w, nr_of_projections=rows, dimx_p=w, dimy_p=n, dimz_p=rows,
                  data_offset=(RSQ_DATA_OFFSET - 512) // 512)
    fields.update(header or {})
    names1 = ["data_type", "nr_of_bytes", "nr_of_blocks", "patient_index", "scanner_id", "creation_date0",
              "creation_date1"]
    names2 = ["dimx_p", "dimy_p", "dimz_p", "dimx_um", "dimy_um", "dimz_um", "slice_thickness_um",
              "slice_increment_um", "slice_1_pos_um", "min_data_value", "max_data_value", "mu_scaling",
              "nr_of_samples", "nr_of_projections", "scandist_um", "scanner_type", "sampletime_us",
              "index_measurement", "site", "reference_line_um", "recon_alg"]
    blk = bytearray(512)
    blk[0:16] = b"CTDATA-HEADER_V1"
    for k, f in enumerate(names1):
        struct.pack_into("<i", blk, 16 + 4 * k, int(fields.get(f, 0)))
    for k, f in enumerate(names2):
        struct.pack_into("<i", blk, 44 + 4 * k, int(fields.get(f, 0)))
    blk[128:168] = name.encode()[:40].ljust(40, b"\0")
    struct.pack_into("<i", blk, 168, int(fields.get("energy", 0)))
    struct.pack_into("<i", blk, 172, int(fields.get("intensity", 0)))
    struct.pack_into("<i", blk, 508, int(fields["data_offset"]))
    head = bytearray(RSQ_DATA_OFFSET)
    head[0:512] = blk
    bh = "Corr at %d %d %d:  %.6f %.6f %.6f" % (*bh_x, *bh_y)
    head[RSQ_BH_OFFSET:RSQ_BH_OFFSET + 152] = bh.encode().ljust(152, b"\0")
    with open(path, "wb") as f:
        f.write(head)
        for r in range(rows):
            f.write(dark[r].tobytes())
            f.write(flat[r].tobytes())
            f.write(counts[r].tobytes())
