"""The header-only C++ FilteredBackProjection (include/tk_fdk.hpp) drives the
library with the reference's own call sequence (FBPG/para_TC.cpp:130-153)."""
import os
import subprocess

import numpy as np
import pytest

from _util import rel_rmse, small_geometry
from tomokvas_gb300.phantom import head_phantom

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(tklib, tmp_path_factory):
    from tomokvas_gb300._build import LIB_DIR

    exe = str(tmp_path_factory.mktemp("cpp") / "para_driver")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
           os.path.join(ROOT, "tests", "cpp", "para_driver.cpp"), "-o", exe, "-L", LIB_DIR, "-ltk_fdk",
           "-Wl,-rpath," + LIB_DIR]
    subprocess.run(cmd, check=True)
    return exe


def run(driver, tmp_path, g, sino):
    src, dst = tmp_path / "sino.f32", tmp_path / "vol.f32"
    np.ascontiguousarray(sino, dtype=np.float32).tofile(src)
    args = [driver, str(src), str(dst)] + [str(v) for v in (g.W, g.N, g.H, g.X, g.Y, g.Z, g.zb, g.D, g.tau, g.dfi,
                                                             g.scale)]
    r = subprocess.run(args, capture_output=True, text=True)
    return r, dst


def test_cpp_driver_builds_and_reports_errors(driver, tmp_path):
    """With an invalid geometry Initialize fails cleanly (no crash) and says why."""
    g = small_geometry(W=32, N=8, H=8, vol=(8, 8, 8)).replace(D=-1.0)
    r, _ = run(driver, tmp_path, g, np.zeros((g.H, g.N, g.W), np.float32))
    assert r.returncode == 1
    assert "tk_fdk" in r.stderr


@pytest.mark.gpu
def test_cpp_driver_reconstructs(orc, cuda, driver, tmp_path):
    g = small_geometry(W=64, N=90, H=64, vol=(48, 48, 40), zb=16)
    G = orc.geom_from(g)
    sino = orc.project_ellipsoids(head_phantom(g.fov_radius_cm * 0.8, seed=3), G, "sino")
    r, dst = run(driver, tmp_path, g, sino)
    assert r.returncode == 0, r.stderr
    assert "Multi-Processors" in r.stdout  # fShowInfo
    vol = np.fromfile(dst, dtype=np.float32).reshape(g.Z, g.Y, g.X)
    assert rel_rmse(vol, orc.fdk_f32(sino, G)) < 1e-5
