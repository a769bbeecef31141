"""Generate the committed golden fixtures from the reference itself.

Run in a checkout that has the reference tree (default /root/reference, or
OH_REFERENCE_ROOT):  python tests/golden/make_golden.py

keti_sample.npz   the reference's own loaders read its sample inputs
                  (example_cpu/TestPointCloud.dat, TestSpec.config); the first
                  64 points are then rendered by the reference's
                  ophGenCghPointCloud (compiled from its sources by
                  oracle/build.py, sequential) on a 256x128 crop of the SLM
                  with the sample's pitch, wavelength and 22.5 deg tilts, and
                  on a 128x96 grid with zero tilt.
keti_synth.npz    config-1 geometry (8 um pitch, 532 nm, points in +-2 mm at
                  z 0.10-0.12 m) on a 128x128 grid with 300 seeded points,
                  rendered by the same compiled reference.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import build as ob  # noqa: E402
from oracle import pointcloud as opc  # noqa: E402
from openholo_gb300 import scenes  # noqa: E402

OUT = Path(__file__).resolve().parent


def main():
    if ob.build_reference() is None:
        raise SystemExit("reference sources not found")
    L = opc._reference()
    ex = ob.REFERENCE_ROOT / "OpenHolo_KETI/VS/Openholo_Generation_PointCloud_Library_beta_v1.0/example_cpu"
    buf = np.zeros((4096, 5), dtype=np.float32)
    n = L.keti_ref_load_points(str(ex / "TestPointCloud.dat").encode(), buf.ctypes.data_as(C.c_void_p), 4096)
    assert n == 1453, n
    s11 = np.zeros(11, dtype=np.float32)
    nxny = np.zeros(2, dtype=np.int32)
    assert L.keti_ref_load_spec(str(ex / "TestSpec.config").encode(), s11.ctypes.data_as(C.c_void_p),
                                nxny.ctypes.data_as(C.c_void_p)) == 1
    pts = buf[:64]
    xyza = np.stack([pts[:, 0], pts[:, 1], pts[:, 2], pts[:, 4]], axis=1).astype(np.float32)
    base = dict(scale_x=float(s11[0]), scale_y=float(s11[1]), scale_z=float(s11[2]), offset_depth=float(s11[3]),
                pitch_x=float(s11[4]), pitch_y=float(s11[5]), tilt_x=float(s11[7]), tilt_y=float(s11[8]))
    base["lambda"] = float(s11[6])
    spec_a = dict(base, nx=256, ny=128)
    spec_b = dict(base, nx=128, ny=96, tilt_x=0.0, tilt_y=0.0)
    out_a = opc.reference_keti(xyza, spec_a)
    out_b = opc.reference_keti(xyza, spec_b)
    np.savez_compressed(OUT / "keti_sample.npz", xyza=xyza, spec11=s11, slm_nxny=nxny,
                        nx_a=256, ny_a=128, fringe_a=out_a, nx_b=128, ny_b=96, fringe_b=out_b,
                        first_rows=buf[:4])
    pts2 = scenes.pointcloud_scene(2024, 300).astype(np.float32)
    spec_c = dict(scale_x=1.0, scale_y=1.0, scale_z=1.0, offset_depth=0.0, pitch_x=8e-6, pitch_y=8e-6,
                  nx=128, ny=128, tilt_x=0.0, tilt_y=0.0)
    spec_c["lambda"] = 532e-9
    np.savez_compressed(OUT / "keti_synth.npz", xyza=pts2, fringe=opc.reference_keti(pts2, spec_c))
    print("wrote", sorted(p.name for p in OUT.glob("*.npz")))


if __name__ == "__main__":
    main()
