"""The reference's own point-cloud GPU kernel, launched as the reference's
host code launches it — TEST INFRASTRUCTURE ONLY (tests/ use it to check the
library against the reference's GPU output and to time it as a baseline).

oracle/build.py compiles OpenHolo_KETI/VS/Openholo_Generation_PointCloud_
Library_beta_v1.0/ophgen_pointcloud_gpu/ophgen_pointcloud_gpu.cpp (from the
reference tree, unchanged) into oracle/_ref/pc_ref.cubin for sm_103a.  This
module fills the kernel's constant block (OphKernelConst,
ophgen_pointcloud_gpu.cpp:367-389) in float as openholo::gpu::
ophGenCghPointCloud_cuda does (:418-466), with its grid rule (:419-429:
blocks of THREAD_X x THREAD_Y = 32 x 16 threads, block counts doubled from
2 until they cover the field) and one launch over all points (:488-491).
The reference leaves dst uninitialised (:484); here it is zeroed first.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

from .dm_reference import _Driver

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "pc_ref.cubin"
KERNEL = "_Z27ophKernelCghPointCloud_cudaP6float3PfPK14OphKernelConstS1_"
THREAD_X, THREAD_Y = 32, 16                    # ophgen_pointcloud_gpu.h:33-34
CUDART_PI_F = np.float32(math.pi)              # pi rounded to float, as the reference writes it


class _ConstBlock(C.Structure):
    """OphKernelConst (ophgen_pointcloud_gpu.cpp:367-389): 14 four-byte fields."""
    _fields_ = [("n_points", C.c_int), ("scaleX", C.c_float), ("scaleY", C.c_float), ("scaleZ", C.c_float),
                ("offsetDepth", C.c_float), ("Nx", C.c_int), ("Ny", C.c_int), ("sin_thetaX", C.c_float),
                ("sin_thetaY", C.c_float), ("k", C.c_float), ("pixel_x", C.c_float), ("pixel_y", C.c_float),
                ("halfLength_x", C.c_float), ("halfLength_y", C.c_float)]


def grid(nx: int, ny: int):
    """The reference's block counts (ophgen_pointcloud_gpu.cpp:419-429)."""
    bx, by = nx // THREAD_X, ny // THREAD_Y
    gx = gy = 2
    while not (gx >= bx and gy >= by):
        if gx < bx:
            gx *= 2
        if gy < by:
            gy *= 2
    return gx, gy


class ReferencePointCloudGPU:
    def __init__(self):
        self.d = _Driver(CUBIN, {"pc": KERNEL})

    def const_block(self, n, spec):
        f = np.float32
        c = _ConstBlock()
        c.n_points = n
        c.scaleX, c.scaleY, c.scaleZ = f(spec["scale_x"]), f(spec["scale_y"]), f(spec["scale_z"])
        c.offsetDepth = f(spec["offset_depth"])
        c.Nx, c.Ny = spec["nx"], spec["ny"]
        tx = f(spec["tilt_x"]) * (CUDART_PI_F / f(180.0))
        ty = f(spec["tilt_y"]) * (CUDART_PI_F / f(180.0))
        c.sin_thetaX, c.sin_thetaY = f(math.sin(tx)), f(math.sin(ty))
        c.k = (f(2.0) * CUDART_PI_F) / f(spec["lambda"])
        c.pixel_x, c.pixel_y = f(spec["pitch_x"]), f(spec["pitch_y"])
        c.halfLength_x = (c.pixel_x * f(c.Nx)) / f(2.0)
        c.halfLength_y = (c.pixel_y * f(c.Ny)) / f(2.0)
        return c

    def launch(self, xyz, amp, cfg, dst):
        """One kernel launch on device tensors: xyz float32 [n][3], amp
        float32 [n], cfg uint8 [56] (the constant block), dst float32
        [ny][nx] (accumulated into, as the reference does)."""
        nx, ny = dst.shape[1], dst.shape[0]
        gx, gy = grid(nx, ny)
        self.d.launch2d("pc", (gx, gy), (THREAD_X, THREAD_Y), xyz.data_ptr(), amp.data_ptr(), cfg.data_ptr(),
                        dst.data_ptr())

    def run(self, pts: np.ndarray, spec: dict):
        """pts: [n][4] x, y, z, amplitude.  Returns the float32 fringe
        [ny][nx] on the device (zeroed, then one launch)."""
        import torch
        n = pts.shape[0]
        xyz = torch.from_numpy(np.ascontiguousarray(pts[:, :3], dtype=np.float32)).cuda()
        amp = torch.from_numpy(np.ascontiguousarray(pts[:, 3], dtype=np.float32)).cuda()
        c = self.const_block(n, spec)
        cfg = torch.frombuffer(bytearray(bytes(c)), dtype=torch.uint8).cuda()
        dst = torch.zeros((spec["ny"], spec["nx"]), dtype=torch.float32, device="cuda")
        self.launch(xyz, amp, cfg, dst)
        return dst, (xyz, amp, cfg)
