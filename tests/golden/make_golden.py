"""Generates the golden fixtures: outputs of the reference's own FDK kernels.

Runs Lukas-kV/TomoKvas FBPG/kernel.cu (compiled by oracle/ref_build.py) with
cuFFT, driven in the reference engine's order by oracle/tk_refrun.cpp, on
seeded analytic phantoms.  Needs a GPU and the prebuilt reference fatbin:

    python tests/golden/make_golden.py [out_dir]

Each fixture stores the geometry, the phantom (ellipsoid records), a checksum
of the projections the reference consumed (regenerated from the phantom by
the oracle's analytic projector at test time) and selected output slices.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from _util import small_geometry  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from oracle import refrun  # noqa: E402
from tomokvas_gb300.geometry import config  # noqa: E402
from tomokvas_gb300.phantom import head_phantom  # noqa: E402

FIELDS = ["W", "N", "H", "cX", "cZ", "dfi", "D", "tau", "X", "Y", "Z", "cx", "cy", "cz", "rot", "scale",
          "dirx", "diry", "dirz", "zb"]


def cases():
    yield "head64", small_geometry(W=64, N=90, H=64, vol=(48, 48, 48), zb=16), 1, None
    yield "w66", small_geometry(W=66, N=60, H=40, vol=(32, 32, 32), zb=16), 2, None
    yield "flips_rot_scale", small_geometry(W=64, N=72, H=70, vol=(40, 40, 40), voxel_mm=1.2, zb=30, dirx=1,
                                            diry=1, dirz=1, rot=0.3), 3, None
    yield "quirk_z33_zb16", small_geometry(W=32, N=24, H=48, vol=(16, 16, 33), zb=16), 4, None
    yield "c1_256", config("c1").replace(zb=16), 21, [40, 128, 230]


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    for name, g, seed, slices in cases():
        G = orc.geom_from(g)
        ell = head_phantom(g.fov_radius_cm * 0.85, seed=seed)
        sino = orc.project_ellipsoids(ell, G, "sino")
        vol = refrun.fdk(sino, g)
        z = np.arange(g.Z) if slices is None else np.asarray(slices)
        np.savez_compressed(os.path.join(out_dir, f"ref_{name}.npz"),
                            geometry=np.array([float(getattr(g, f)) for f in FIELDS]),
                            fields=np.array(FIELDS), ellipsoids=ell, slices=z.astype(np.int32),
                            volume=vol[z].astype(np.float32),
                            sino_checksum=np.array([float(np.sum(sino, dtype=np.float64)),
                                                    float(np.sum(np.square(sino, dtype=np.float64)))]))
        print(name, vol.shape, float(np.abs(vol).max()))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
