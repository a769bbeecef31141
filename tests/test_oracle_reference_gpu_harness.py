"""Host-side pieces of the reference-GPU harnesses (no GPU needed): the
point-cloud kernel's grid rule and constant block follow the reference's
host function (OpenHolo_KETI/.../ophgen_pointcloud_gpu/ophgen_pointcloud_gpu.cpp:
418-466, OphKernelConst at :367-389)."""
import ctypes as C
import math

import numpy as np

from oracle import pc_reference_gpu as pref


def test_grid_rule_covers_the_field_with_doubled_block_counts():
    # blocks of 32 x 16 threads; both counts start at 2 and double until they
    # cover nx / 32 and ny / 16 (the two loops advance together)
    assert pref.grid(1024, 1024) == (32, 64)
    assert pref.grid(1920, 1080) == (64, 128)     # 60 -> 64, 67 -> 128
    assert pref.grid(64, 32) == (2, 2)
    for nx, ny in ((256, 320), (4096, 2160), (100, 50)):
        gx, gy = pref.grid(nx, ny)
        assert gx * 32 >= nx // 32 * 32 and gy * 16 >= ny // 16 * 16
        assert gx & (gx - 1) == 0 and gy & (gy - 1) == 0


def test_constant_block_layout_and_values():
    assert C.sizeof(pref._ConstBlock) == 56
    spec = {"scale_x": 1.0, "scale_y": 2.0, "scale_z": 0.5, "offset_depth": 0.01, "pitch_x": 8e-6, "pitch_y": 6e-6,
            "nx": 1024, "ny": 768, "lambda": 532e-9, "tilt_x": 1.5, "tilt_y": -2.0}
    c = pref.ReferencePointCloudGPU.const_block(None, 5000, spec)
    f = np.float32
    assert c.n_points == 5000 and c.Nx == 1024 and c.Ny == 768
    assert c.scaleY == f(2.0) and c.offsetDepth == f(0.01)
    # float arithmetic as the reference's host code does it
    assert c.k == f(f(2.0) * f(math.pi) / f(532e-9))
    assert c.halfLength_x == f(f(8e-6) * f(1024) / f(2.0))
    assert c.sin_thetaX == f(math.sin(f(1.5) * (f(math.pi) / f(180.0))))
    raw = bytes(c)
    assert np.frombuffer(raw[:4], dtype=np.int32)[0] == 5000
    assert np.frombuffer(raw[20:28], dtype=np.int32).tolist() == [1024, 768]
