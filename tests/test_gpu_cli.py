"""The para_TC-equivalent driver end to end on the GPU: setting.xml + .CRA +
raw projections in, .bin/.siz out (tomokvas_gb300/lib/tk_para_tc).

Two scan blocks with different centres of rotation, counter-clockwise and
clockwise storage, a vertical detector offset and an axis flip from
setting.xml.  Each scan block's slab of the .bin volume must match the FP64
oracle of the geometry the reference's driver derives from the same header
(noise-free analytic projections): relative RMSE <= 1e-5.
"""
import os
import subprocess

import numpy as np
import pytest

from _util import rel_rmse
from tomokvas_gb300 import _build
from tomokvas_gb300.phantom import head_phantom
from tomokvas_gb300.scanfile import cra_geometry, read_binsiz, write_cra

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("clockwise,xdir", [(False, 0), (True, 1)])
def test_cli_reconstructs_cra_scan(orc, cuda, tmp_path, clockwise, xdir):
    W, H, N = 64, 48, 60
    spacing_um, distance_cm, rot_deg, voff = 20.0, 1.0, 7.0, 0.5  # D = 500 px
    centres = [31.5, 32.25]
    (tmp_path / "setting.xml").write_text(
        '<GPU_FBP>\n    <GPU ID="0" MemLimit_MiB="1848" AllocLimit_MiB="1024" />\n'
        f'    <RECONSTRUCTION SimultaneouslyReconstructedSlices="16" X_direction="{xdir}" Y_direction="0" '
        f'Z_direction="0" DetectorVerticalCenterOffset="{voff}" />\n    <GENERAL WaitForEnter="0" />\n</GPU_FBP>\n')
    geos, projs, ells = [], [], []
    for k, c in enumerate(centres):
        g = cra_geometry(spacing_um, distance_cm, W, H, N, c, rot_deg, clockwise, x_dimension=40, z_dimension=40,
                         vertical_offset=voff, dirs=(xdir, 0, 0))
        G = orc.geom_from(g)
        ell = head_phantom(g.fov_radius_cm * 0.8, seed=40 + k)
        projs.append(orc.project_ellipsoids(ell, G, "proj"))  # [N][H][W], increasing angle
        geos.append((g, G))
    write_cra(str(tmp_path), "scan", np.stack(projs), spacing_um, distance_cm, centres, rotate_angle_deg=rot_deg,
              clockwise=clockwise, x_dimension=40, z_dimension=40)
    exe = _build.build_cli()
    subprocess.run([exe, "--quiet", str(tmp_path / "scan.CRA")], cwd=tmp_path, check=True, timeout=300)
    vol = read_binsiz(str(tmp_path), "scan")
    g0 = geos[0][0]
    assert vol.shape == (2 * g0.Z, g0.Y, g0.X)
    for k, (g, G) in enumerate(geos):
        ref = orc.fdk_f64(np.ascontiguousarray(np.transpose(projs[k], (1, 0, 2))), G)
        assert rel_rmse(vol[k * g.Z:(k + 1) * g.Z], ref) < 1e-5
