"""Point-light-source summation with the shape of CWO++'s cwoPLS class
(OpenHolo_WRP/openwrp_console_ver 1.0/cwo/src/cwoPLS.cpp): a point buffer of
cwoObjPoint records (a_re, a_im, x, y, z), destination pitch/offset, source
offset and wavelength, and the three per-pixel sums Huygens(z, ph),
Fresnel(z, ph) and CGHFresnel(z, ph).  Results are device tensors (complex
field, or real intensity for CGHFresnel); every call runs oh_pls.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib


class PointLightSources:
    def __init__(self, ctx: _lib.Context, nx: int, ny: int, pitch=(8e-6, 8e-6), lam=532e-9,
                 dst_offset=(0.0, 0.0), src_offset=(0.0, 0.0), precision="fp32", engine=_lib.PLS_ENGINE_AUTO,
                 use_amplitude=False):
        self.ctx, self.nx, self.ny = ctx, nx, ny
        self.pitch, self.lam = pitch, lam
        self.dst_offset, self.src_offset = dst_offset, src_offset
        self.precision, self.engine, self.use_amplitude = precision, engine, use_amplitude
        self.points = None

    def set_points(self, points) -> None:
        """points: (n, 5) float32 array or tensor of (a_re, a_im, x, y, z)."""
        t = torch.as_tensor(points, dtype=torch.float32).reshape(-1, 5).contiguous()
        self.points = t.cuda()

    def _run(self, mode: int, z: float, ph: float) -> torch.Tensor:
        if self.points is None:
            raise ValueError("no points: call set_points first")
        fp64 = self.precision == "fp64"
        if mode == _lib.PLS_CGH_FRESNEL:
            out = torch.empty((self.ny, self.nx), dtype=torch.float64 if fp64 else torch.float32, device="cuda")
        else:
            out = torch.empty((self.ny, self.nx), dtype=torch.complex128 if fp64 else torch.complex64, device="cuda")
        p = _lib.PlsParams(self.nx, self.ny, self.pitch[0], self.pitch[1], self.dst_offset[0], self.dst_offset[1],
                           self.src_offset[0], self.src_offset[1], self.lam, z, ph, mode,
                           1 if self.use_amplitude else 0, self.engine)
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.call("oh_pls", self.ctx.handle, 1 if fp64 else 0, C.byref(p), C.c_void_p(self.points.data_ptr()),
                  self.points.shape[0], C.c_void_p(out.data_ptr()), st)
        return out

    def Huygens(self, z: float, ph: float = 0.0) -> torch.Tensor:
        return self._run(_lib.PLS_HUYGENS, z, ph)

    def Fresnel(self, z: float, ph: float = 0.0) -> torch.Tensor:
        return self._run(_lib.PLS_FRESNEL, z, ph)

    def CGHFresnel(self, z: float, ph: float = 0.0) -> torch.Tensor:
        return self._run(_lib.PLS_CGH_FRESNEL, z, ph)
