"""Pin the point-cloud oracle: its FP32 restatement of ophGenCghPointCloud
equals the reference's own compiled output bit for bit (committed fixtures
made by tests/golden/make_golden.py, and the live reference build when the
reference tree is present); its FP64 form agrees with that to the
reference's FP32 phase noise."""
from pathlib import Path

import numpy as np
import pytest

from oracle import pointcloud as opc
from oracle import wrp as owrp

GOLD = Path(__file__).resolve().parent / "golden"


def _spec(s11, nx, ny, tilt):
    d = dict(scale_x=float(s11[0]), scale_y=float(s11[1]), scale_z=float(s11[2]), offset_depth=float(s11[3]),
             pitch_x=float(s11[4]), pitch_y=float(s11[5]), nx=nx, ny=ny, tilt_x=tilt[0], tilt_y=tilt[1])
    d["lambda"] = float(s11[6])
    return d


def test_keti_restatement_matches_reference_fixture():
    g = np.load(GOLD / "keti_sample.npz")
    s11 = g["spec11"]
    a = opc.keti_f32(g["xyza"], _spec(s11, int(g["nx_a"]), int(g["ny_a"]), (float(s11[7]), float(s11[8]))))
    assert np.array_equal(a, g["fringe_a"])
    b = opc.keti_f32(g["xyza"], _spec(s11, int(g["nx_b"]), int(g["ny_b"]), (0.0, 0.0)))
    assert np.array_equal(b, g["fringe_b"])


def test_keti_synthetic_fixture():
    g = np.load(GOLD / "keti_synth.npz")
    s = dict(scale_x=1.0, scale_y=1.0, scale_z=1.0, offset_depth=0.0, pitch_x=8e-6, pitch_y=8e-6, nx=128, ny=128,
             tilt_x=0.0, tilt_y=0.0)
    s["lambda"] = 532e-9
    assert np.array_equal(opc.keti_f32(g["xyza"], s), g["fringe"])
    exact = opc.pc_f64(g["xyza"].astype(np.float64), s).real
    err = np.linalg.norm(g["fringe"] - exact) / np.linalg.norm(exact)
    assert 1e-3 < err < 0.5        # the reference's FP32 phase noise at k r ~ 1.2e6 rad


def test_keti_live_reference_when_present():
    if not opc.reference_available():
        pytest.skip("reference tree not present")
    rng = np.random.default_rng(0)
    xyza = np.concatenate([rng.uniform(-1, 1, (40, 2)), rng.uniform(-1.2, -1.0, (40, 1)), rng.uniform(0, 1, (40, 1))],
                          axis=1).astype(np.float32)
    s = dict(scale_x=0.05, scale_y=0.05, scale_z=0.05, offset_depth=0.06, pitch_x=4.62e-7, pitch_y=4.62e-7, nx=96,
             ny=64, tilt_x=22.5, tilt_y=-5.0)
    s["lambda"] = 5.32e-7
    assert np.array_equal(opc.keti_f32(xyza, s), opc.reference_keti(xyza, s))


def test_fresnel_conv_vs_transfer_function():
    """The conv-form (CWO) and transfer-function-form (MATLAB) Fresnel
    propagators agree on a well-sampled, band-limited field."""
    n, dp, lam, z = 128, 8e-6, 532e-9, 0.01
    y, x = np.mgrid[0:n, 0:n] - n / 2
    U = np.exp(-(x ** 2 + y ** 2) / (2 * 6.0 ** 2)).astype(np.complex128)
    a = owrp.fresnel_conv(U, dp, lam, z)
    Up = np.zeros((2 * n, 2 * n), np.complex128)
    Up[n // 2:n // 2 + n, n // 2:n // 2 + n] = U
    b = owrp.fresnel_tf(Up, dp, dp, z, lam)[n // 2:n // 2 + n, n // 2:n // 2 + n]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-2
