"""The OPHWRP drop-in (include/oh_openholo_wrp.hpp): a program written the way
the reference's openwrp.cpp drives the class builds against liboh_gb300.so and
reproduces the oracle's WRP plane and propagated hologram."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import pointcloud as opc
from oracle import wrp as owrp

ROOT = Path(__file__).resolve().parents[1]
LIBDIR = ROOT / "openholo_gb300"


def _compile(src, out):
    cmd = ["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(src), "-o", str(out),
           "-L", str(LIBDIR), "-loh_gb300", f"-Wl,-rpath,{LIBDIR}"]
    return subprocess.run(cmd, capture_output=True, text=True)


def test_dropin_program_builds(lib_built, tmp_path):
    r = _compile(ROOT / "tests/cpp/wrp_dropin.cpp", tmp_path / "wrp_dropin")
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.gpu
def test_dropin_matches_oracle(lib_built, tmp_path):
    from openholo_gb300 import scenes
    res, dp, lam = 129, 8e-6, 532e-9
    pts = scenes.wrp_scene(31, 150, box=(0.8e-3, 0.8e-3, 0.1e-3), zc=0.0)
    txt = tmp_path / "object.txt"
    txt.write_text("".join(f"{x:.9g} {y:.9g} {z:.9g}\n" for x, y, z in pts))
    exe = tmp_path / "wrp_dropin"
    r = _compile(ROOT / "tests/cpp/wrp_dropin.cpp", exe)
    assert r.returncode == 0, r.stderr[-2000:]
    run = subprocess.run([str(exe), str(txt), str(tmp_path / "out")], capture_output=True, text=True)
    assert run.returncode == 0, (run.returncode, run.stdout + run.stderr)
    wrp = np.fromfile(tmp_path / "out_wrp.c64", dtype=np.complex64).reshape(res, res)
    holo = np.fromfile(tmp_path / "out_holo.c64", dtype=np.complex64).reshape(res, res)
    # the class reads the points into float, as the reference does
    pts32 = np.loadtxt(txt).astype(np.float32).astype(np.float64)
    z = float(np.float32(0.5e-3))
    ref_wrp = opc.wrp_f64(pts32, res, res, float(np.float32(dp)), float(np.float32(lam)), z, 0)
    assert np.linalg.norm(wrp - ref_wrp) <= 1e-4 * np.linalg.norm(ref_wrp)
    ref_holo = owrp.fresnel_conv(wrp.astype(np.complex128), float(np.float32(dp)), float(np.float32(lam)),
                                 float(np.float32(0.05)))
    assert np.linalg.norm(holo - ref_holo) <= 1e-4 * np.linalg.norm(ref_holo)
    for name in ("out_wrp_table.bmp", "out_wrp_result.bmp"):
        assert (tmp_path / name).stat().st_size == 54 + 1024 + ((res + 3) & ~3) * res
