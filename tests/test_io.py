"""Host-side scan and volume formats (include/tk_io.hpp), no GPU.

A C++ program (tests/cpp/io_check.cpp) built with g++ reads .CRA scans
written by tomokvas_gb300.scanfile and writes .bin/.siz volumes; the
derived geometry is compared with a restatement of cra_con's float/int
arithmetic (FBPG/mucat_file.cpp:139-161), the loaded frames with the data
written (clockwise scans reversed, second scan block offset), the volume
file with the values written (two passes, the second collecting), and
setting.xml parsing with LoadSetting's defaults (FBPG/para_TC.cpp:180-260),
and .RSQ raw scans: the header block, the beam-hardening line A, B
(FBPG/rsq_load.cpp:538-542) and the per-row dark, flat and projection rows
(FBPG/rsq_load.cpp:185-227, 299-325).
"""
import json
import math
import os
import subprocess

import numpy as np
import pytest

from tomokvas_gb300.scanfile import cra_derived, read_binsiz, write_cra, write_rsq

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def io_check(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("io") / "io_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-pthread", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "io_check.cpp"), "-o", exe], check=True)
    return exe


def run(exe, *args):
    out = subprocess.run([exe, *map(str, args)], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


def frames(blocks, N, H, W, seed=0):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(blocks, N, H, W)).astype(np.float32)


@pytest.mark.parametrize("clockwise,crlf", [(False, False), (True, True)])
def test_cra_header_and_frames(io_check, tmp_path, clockwise, crlf):
    blocks, N, H, W = 2, 12, 10, 16
    p = frames(blocks, N, H, W, seed=1)
    write_cra(str(tmp_path), "scan", p, sample_spacing_um=7.5, distance_cm=1.25, centres=[7.25, 8.5],
              rotate_angle_deg=12.0, clockwise=clockwise, x_dimension=14, z_dimension=8, scale=0.5, crlf=crlf)
    for blk in range(blocks):
        r = run(io_check, "cra", tmp_path, "scan", blk, tmp_path / "p.f32", tmp_path / "s.f32")
        assert r["rc"] == 0 and r["load"] == [0, 0]
        dist, dfi, xd, zd = cra_derived(7.5, 1.25, W, H, N, 14, 8)
        assert r["distance"] == np.float32(dist) and r["dfi"] == np.float32(dfi)
        assert r["rec"] == [xd, xd, zd] and r["size"] == [W, N, H] and r["blocks"] == blocks
        assert r["centre"] == [7.25, 8.5][blk] and r["scale"] == 0.5 and r["sampling"] == 7.5
        rot = (float(np.float32(dfi)) if clockwise else 0.0) + 12.0 * math.pi / 180.0
        assert r["rot"] == pytest.approx(rot, rel=1e-15) and r["clockwise"] == int(clockwise)
        got_p = np.fromfile(tmp_path / "p.f32", dtype=np.float32).reshape(N, H, W)
        got_s = np.fromfile(tmp_path / "s.f32", dtype=np.float32).reshape(H, N, W)
        np.testing.assert_array_equal(got_p, p[blk])                       # projection-major, increasing angle
        np.testing.assert_array_equal(got_s, np.transpose(p[blk], (1, 0, 2)))  # the reference's [H][N][W]


def test_cra_clamps_and_missing_file(io_check, tmp_path):
    # x_dimension 0 -> the FOV width, z_dimension clamped to (D - X/2)/D * H made even
    p = frames(1, 4, 64, 256)
    write_cra(str(tmp_path), "clamp", p, sample_spacing_um=50.0, distance_cm=0.5, centres=[127.5],
              z_dimension=1000)
    r = run(io_check, "cra", tmp_path, "clamp", 0, tmp_path / "p.f32", tmp_path / "s.f32")
    dist, _, xd, zd = cra_derived(50.0, 0.5, 256, 64, 4, 0, 1000)
    assert dist == 100.0 and r["rec"] == [xd, xd, zd]
    assert zd % 2 == 0 and zd < 64 and xd < 256
    assert run(io_check, "cra", tmp_path, "absent", 0, tmp_path / "p.f32", tmp_path / "s.f32")["rc"] == -1


@pytest.mark.parametrize("Z,zb,sb", [(10, 4, 1), (9, 3, 2), (5, 16, 1)])
def test_binsiz_blocks_and_collecting(io_check, tmp_path, Z, zb, sb):
    X, Y = 6, 5
    assert run(io_check, "binsiz", tmp_path, "vol", X, Y, Z, zb, sb)["errors"] == 0
    vol = read_binsiz(str(tmp_path), "vol")
    assert vol.shape == (Z * sb, Y, X)
    with open(tmp_path / "vol.siz") as f:
        assert f.read() == f"{X} {Y} {Z * sb} 0"
    i = np.arange(X * Y, dtype=np.float32).reshape(Y, X)
    for s in range(sb):
        for z in range(Z):
            want = np.float32(1000 * s + z) + np.float32(0.001) * i + np.float32(0.5)
            np.testing.assert_allclose(vol[s * Z + z], want, rtol=0, atol=1e-3)


def test_settings(io_check, tmp_path):
    x = tmp_path / "setting.xml"
    x.write_text('<GPU_FBP>\n    <GPU ID="3" MemLimit_MiB="1848" AllocLimit_MiB="512" />\n'
                 '    <RECONSTRUCTION SimultaneouslyReconstructedSlices="30" X_direction="1" Y_direction="0" '
                 'Z_direction="2" DetectorVerticalCenterOffset="-1.5" />\n    <GENERAL WaitForEnter="0" />\n'
                 '</GPU_FBP>\n')
    r = run(io_check, "settings", x, tmp_path / "saved.xml")
    assert r == {"found": 1, "GPUId": 3, "GPUmemLimit": 1848, "GPUAllocLimit": 512, "VerticalCenter": -1.5,
                 "NoOfSlicesInOneBlock": 30, "x": 1, "y": 0, "z": 1, "WaitForEnter": 0}
    r2 = run(io_check, "settings", tmp_path / "saved.xml")
    assert r2 == r
    # no file: LoadSetting's defaults
    d = run(io_check, "settings", tmp_path / "none.xml")
    assert d == {"found": 0, "GPUId": 0, "GPUmemLimit": 5120, "GPUAllocLimit": 1024, "VerticalCenter": 0,
                 "NoOfSlicesInOneBlock": 16, "x": 0, "y": 0, "z": 0, "WaitForEnter": 1}


def test_rsq_header_beam_hardening_and_rows(io_check, tmp_path):
    rows, N, W = 5, 12, 16
    rng = np.random.default_rng(7)
    counts = rng.integers(100, 60000, size=(rows, N, W), dtype=np.uint16)
    dark = rng.integers(0, 50, size=(rows, W), dtype=np.uint16)
    flat = rng.integers(50000, 65000, size=(rows, W), dtype=np.uint16)
    path = tmp_path / "scan.rsq"
    write_rsq(str(path), counts, dark, flat, bh_x=(120, 260, 410), bh_y=(0.85, 1.9, 3.2),
              name="phantom", header=dict(energy=45000, dimz_um=777))
    r = run(io_check, "rsq", path, W, N, 1, 3, tmp_path / "raw.u16", tmp_path / "d.f32", tmp_path / "f.f32")
    assert r["rc"] == 0 and r["load"] == 0 and r["sinograms"] == rows
    assert r["check"] == "CTDATA-HEADER_V1" and r["name"] == "phantom" and r["energy"] == 45000
    assert r["samples"] == W and r["projections"] == rows and r["dim"] == [W, N, rows]
    assert r["bh_parsed"] == 1 and r["bh_x"] == [120, 260, 410] and r["bh_y"] == [0.85, 1.9, 3.2]
    A = (3.2 - 0.85) / (410 - 120)  # the line through the first and third points
    assert r["A"] == pytest.approx(A, rel=1e-15) and r["B"] == pytest.approx(0.85 - A * 120, rel=1e-15)
    raw = np.fromfile(tmp_path / "raw.u16", dtype=np.uint16).reshape(3, N, W)
    np.testing.assert_array_equal(raw, counts[1:4])  # rows 1..3, sinogram-major [H][N][W]
    np.testing.assert_array_equal(np.fromfile(tmp_path / "d.f32", dtype=np.float32).reshape(3, W), dark[1:4])
    np.testing.assert_array_equal(np.fromfile(tmp_path / "f.f32", dtype=np.float32).reshape(3, W), flat[1:4])
    bad = run(io_check, "rsq", path, W, N, 2, rows, tmp_path / "x", tmp_path / "y", tmp_path / "z")
    assert bad["load"] == -1  # past the last row
    assert run(io_check, "rsq", tmp_path / "absent.rsq", W, N, 0, 0, "a", "b", "c")["rc"] == -1
