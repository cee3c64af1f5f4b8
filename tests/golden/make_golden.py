"""Generates the golden fixtures: outputs of the reference's own FDK kernels.

Runs Lukas-kV/TomoKvas FBPG/kernel.cu (compiled by oracle/ref_build.py) with
cuFFT, driven in the reference engine's order by oracle/tk_refrun.cpp, on
seeded analytic phantoms.  Needs a GPU and the prebuilt reference fatbin:

    python tests/golden/make_golden.py [out_dir]
    python tests/golden/make_golden.py --c2 [out_dir]   (the 1024^3 workload, c2ref_1024.npz, with FP64)

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


C2_SLICES = [0, 480, 512, 544, 1010]
C2_STEP = 4  # every 4th voxel of x and y in the stored slices (1 MB)


def main_c2(out_dir):
    """The 1024^3 workload from 720 x 1024^2 projections (the headline geometry) with the reference's
    own Ram-Lak filter: noise-free line integrals of a seeded 40-ellipsoid phantom, made by this
    repository's GPU projector (tk_phantom_project; a test regenerates them the same way and checks
    the checksum), Z blocks of 16 slices.  Stores five slices at every 4th voxel."""
    import torch

    from tomokvas_gb300 import _lib, device
    from tomokvas_gb300.phantom import random_ellipsoids

    g = config("c2").replace(zb=16)
    ell = random_ellipsoids(40, g.fov_radius_cm, g.Z * g.voxel_cm / 2, seed=11)
    torch.cuda.set_device(0)
    sino = device.phantom_project(g, ell, _lib.TK_LAYOUT_SINOGRAM).cpu().numpy()
    torch.cuda.empty_cache()
    vol = refrun.fdk(sino, g)
    z = np.asarray(C2_SLICES)
    # the FP64 oracle on the same slices: how far the reference's own FP32 pipeline sits from it
    f64 = orc.fdk_f64(sino, orc.geom_from(g), "ramlak", z.astype(np.int32))[:, ::C2_STEP, ::C2_STEP]
    np.savez_compressed(os.path.join(out_dir, "c2ref_1024.npz"), fp64=f64.astype(np.float64),
                        geometry=np.array([float(getattr(g, f)) for f in FIELDS]),
                        fields=np.array(FIELDS), ellipsoids=ell, slices=z.astype(np.int32),
                        step=np.int32(C2_STEP),
                        volume=np.ascontiguousarray(vol[z][:, ::C2_STEP, ::C2_STEP]).astype(np.float32),
                        sino_checksum=np.array([float(np.sum(sino, dtype=np.float64)),
                                                float(np.sum(np.square(sino, dtype=np.float64)))]))
    print("c2_1024", vol.shape, float(np.abs(vol).max()))


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    out = args[0] if args else os.path.dirname(os.path.abspath(__file__))
    if "--c2" in sys.argv:
        main_c2(out)
    else:
        main(out)
