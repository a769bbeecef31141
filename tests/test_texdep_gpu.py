"""oh_texdep_wrp (cwoTexDep::WRP) against the per-texel scatter oracle."""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, scenes
from openholo_gb300._lib import OhError, TexdepParams
from oracle import texdep as otd

pytestmark = pytest.mark.gpu


def _images(ny, nx, seed):
    u = scenes.uniform(seed, 1, 2 * ny * nx).reshape(2, ny, nx)
    tex = (u[0] * 256).astype(np.uint8)
    tex[u[0] < 0.3] = 0                       # texels that add nothing
    dep = (u[1] * 256).astype(np.uint8)
    return tex, dep


def _run(ctx, prec, mode, p, tex, dep):
    cdt = torch.complex128 if prec == "fp64" else torch.complex64
    out = torch.zeros((p.ny, p.nx), dtype=cdt, device="cuda")
    tt = torch.from_numpy(tex).cuda()
    td = torch.from_numpy(dep).cuda() if dep is not None else None
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("oh_texdep_wrp", ctx.handle, 1 if prec == "fp64" else 0, mode, C.byref(p), C.c_void_p(tt.data_ptr()),
              C.c_void_p(td.data_ptr()) if td is not None else None, C.c_void_p(out.data_ptr()), st)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("z", [1e-3, -2.5e-3])
def test_single(ctx, z):
    tex, _ = _images(40, 56, 3)
    p = TexdepParams(56, 40, 8e-6, 6e-6, 532e-9, z, 0.0, 0, 256, 1)
    ref = otd.wrp_single(tex, 8e-6, 6e-6, 532e-9, z)
    assert _rel(_run(ctx, "fp64", _lib.TEXDEP_SINGLE, p, tex, None), ref) < 1e-10
    assert _rel(_run(ctx, "fp32", _lib.TEXDEP_SINGLE, p, tex, None), ref) < 1e-5


@pytest.mark.parametrize("dep_from_texture,with_dep,lo,hi", [(1, True, 0, 256), (0, True, 40, 200), (0, False, 0, 5)])
def test_range(ctx, dep_from_texture, with_dep, lo, hi):
    tex, dep = _images(36, 48, 5)
    z, step = 1e-3, 2e-5
    p = TexdepParams(48, 36, 8e-6, 8e-6, 532e-9, z, step, lo, hi, dep_from_texture)
    d = dep if with_dep else None
    ref = otd.wrp_range(tex, d, 8e-6, 8e-6, 532e-9, z, step, lo, hi, dep_from_texture=bool(dep_from_texture))
    assert _rel(_run(ctx, "fp64", _lib.TEXDEP_RANGE, p, tex, d), ref) < 1e-10
    assert _rel(_run(ctx, "fp32", _lib.TEXDEP_RANGE, p, tex, d), ref) < 1e-5


def test_rejects_bad_arguments(ctx):
    p = TexdepParams(8, 8, 8e-6, 8e-6, 20e-6, 1e-3, 0.0, 0, 256, 1)        # wavelength above 2 pitch
    out = torch.zeros((8, 8), dtype=torch.complex64, device="cuda")
    tex = torch.zeros((8, 8), dtype=torch.uint8, device="cuda")
    with pytest.raises(OhError):
        _lib.call("oh_texdep_wrp", ctx.handle, 0, 0, C.byref(p), C.c_void_p(tex.data_ptr()), None,
                  C.c_void_p(out.data_ptr()), None)
