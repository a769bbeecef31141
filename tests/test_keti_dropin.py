"""The C++ drop-in of the KETI point-cloud API: a program written against
include/oh_openholo_pointcloud.hpp the way the reference's examples are
written links against liboh_gb300.so and reproduces the oracle; and the
reference's own example_cpu.cpp links against the library unchanged."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import encoding as oenc
from oracle import pointcloud as opc

ROOT = Path(__file__).resolve().parents[1]
LIBDIR = ROOT / "openholo_gb300"
EXAMPLE = Path("/root/reference/OpenHolo_KETI/VS/Openholo_Generation_PointCloud_Library_beta_v1.0/example_cpu/"
               "example_cpu.cpp")


def _compile(src, out, extra=()):
    cmd = ["g++", "-std=c++17", "-O2", *extra, "-I", str(ROOT / "include"), str(src), "-o", str(out),
           "-L", str(LIBDIR), "-loh_gb300", f"-Wl,-rpath,{LIBDIR}"]
    return subprocess.run(cmd, capture_output=True, text=True)


def test_reference_example_links_against_library(lib_built, tmp_path):
    if not EXAMPLE.exists():
        pytest.skip("reference tree not present")
    r = _compile(EXAMPLE, tmp_path / "example_cpu", extra=("-fpermissive", "-w"))
    assert r.returncode == 0, r.stderr[-2000:]


def _write_inputs(tmp_path, pts, nx, ny):
    dat = tmp_path / "pts.dat"
    with open(dat, "w") as f:
        f.write(f"{len(pts)}\n")
        for i, (x, y, z, a) in enumerate(pts):
            f.write(f"{i}\t{x:.9g} {y:.9g} {z:.9g} 0.5 {a:.9g}\n")
    cfg = tmp_path / "spec.config"
    vals = [("ScalingXofPointCloud", 1), ("ScalingYofPointCloud", 1), ("ScalingZofPointCloud", 1),
            ("OffsetInDepth", 0), ("SLMpixelPitchX", 8e-6), ("SLMpixelPitchY", 8e-6), ("SLMpixelNumX", nx),
            ("SLMpixelNumY", ny), ("BandpassFilterShape", "circle"), ("BandpassFilterWidthX", 5),
            ("BandpassFilterWidthY", 3), ("FocalLengthofInputLens", 200), ("FocalLengthofOutputLens", 200),
            ("FocalLengthofEyepieceLens", 75), ("WavelengthofLaser", 5.32e-7), ("TiltAngleX", 10),
            ("TiltAngleY", -5)]
    cfg.write_text("".join(f"{k} = {v}\n" for k, v in vals))
    return dat, cfg


@pytest.mark.gpu
def test_dropin_program_matches_oracle(lib_built, tmp_path):
    from openholo_gb300 import scenes
    nx, ny = 96, 64
    pts = scenes.pointcloud_scene(8, 200).astype(np.float32)
    dat, cfg = _write_inputs(tmp_path, pts, nx, ny)
    exe = tmp_path / "keti_dropin"
    r = _compile(ROOT / "tests/cpp/keti_dropin.cpp", exe)
    assert r.returncode == 0, r.stderr[-2000:]
    run = subprocess.run([str(exe), str(dat), str(cfg), str(tmp_path / "out")], capture_output=True, text=True)
    assert run.returncode == 0, run.stdout + run.stderr
    fr = np.fromfile(tmp_path / "out_fringe.f32", dtype=np.float32).reshape(ny, nx)
    frg = np.fromfile(tmp_path / "out_fringe_gpu.f32", dtype=np.float32).reshape(ny, nx)
    spec = dict(scale_x=1.0, scale_y=1.0, scale_z=1.0, offset_depth=0.0, pitch_x=8e-6, pitch_y=8e-6, nx=nx, ny=ny,
                tilt_x=10.0, tilt_y=-5.0)
    spec["lambda"] = np.float32(5.32e-7).item()
    # the program read the points back from text: use the same parsed values
    pts_read = np.loadtxt(dat, skiprows=1)[:, [1, 2, 3, 5]].astype(np.float32)
    exact = opc.pc_f64(pts_read.astype(np.float64), spec).real
    assert np.linalg.norm(fr - exact) / np.linalg.norm(exact) < 1e-3
    assert np.array_equal(fr, frg)
    img = np.fromfile(tmp_path / "out_img.u8", dtype=np.uint8).reshape(ny, nx)
    assert np.abs(img.astype(int) - oenc.keti_normalize(fr).astype(int)).max() <= 1
    assert (tmp_path / "out_img.bmp").stat().st_size == 54 + 1024 + nx * ny
