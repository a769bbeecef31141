"""oh_pls (cwoPLS Huygens / Fresnel / CGHFresnel) against the FP64 oracle."""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, scenes
from openholo_gb300._lib import OhError, PlsParams
from openholo_gb300.pls import PointLightSources
from oracle import pls as opls

pytestmark = pytest.mark.gpu

MODES = {_lib.PLS_HUYGENS: opls.HUYGENS, _lib.PLS_FRESNEL: opls.FRESNEL, _lib.PLS_CGH_FRESNEL: opls.CGH_FRESNEL}
TOL_F32 = 2e-5      # FP32 (phases exact to 2^-23 turn, FP32 sums)
TOL_TENSOR = 1e-4   # split-BF16 tensor-core products
TOL_F64 = 1e-10


def _run(ctx, prec, p, pts):
    fp64 = prec == "fp64"
    if p.mode == _lib.PLS_CGH_FRESNEL:
        out = torch.empty((p.ny, p.nx), dtype=torch.float64 if fp64 else torch.float32, device="cuda")
    else:
        out = torch.empty((p.ny, p.nx), dtype=torch.complex128 if fp64 else torch.complex64, device="cuda")
    t = torch.from_numpy(np.ascontiguousarray(pts, np.float32)).cuda()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("oh_pls", ctx.handle, 1 if fp64 else 0, C.byref(p), C.c_void_p(t.data_ptr()), t.shape[0],
              C.c_void_p(out.data_ptr()), st)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _ref(p, pts):
    return opls.pls(pts, p.nx, p.ny, p.dst_px, p.dst_py, p.lambda_, p.z, p.phase, MODES[p.mode],
                    p.dst_ox, p.dst_oy, p.src_ox, p.src_oy, bool(p.use_amplitude))


@pytest.mark.parametrize("mode", [_lib.PLS_HUYGENS, _lib.PLS_FRESNEL, _lib.PLS_CGH_FRESNEL])
@pytest.mark.parametrize("engine", [_lib.PLS_ENGINE_DIRECT, _lib.PLS_ENGINE_GEMM, _lib.PLS_ENGINE_AUTO])
@pytest.mark.parametrize("use_amp", [0, 1])
def test_pls_matches_oracle(ctx, mode, engine, use_amp):
    # odd width (nx >> 1), offsets on both sides, a phase offset, points off the grid
    pts = scenes.pls_scene(3, 700, xy_half=0.4e-3, z_range=(0.02, 0.03))
    p = PlsParams(97, 64, 8e-6, 6e-6, 1.5e-5, -2.5e-5, 3e-6, -1e-6, 532e-9, 0.004, 0.7, mode, use_amp, engine)
    ref = _ref(p, pts)
    got = _run(ctx, "fp32", p, pts)
    tol = TOL_TENSOR if engine == _lib.PLS_ENGINE_AUTO and mode != _lib.PLS_HUYGENS else TOL_F32
    assert _rel(got, ref) < tol
    got64 = _run(ctx, "fp64", p, pts)
    assert _rel(got64, ref) < TOL_F64


def test_pls_config1_shape_engines_agree(ctx):
    """1024x1024, 5000 points (z 0.10-0.12 m, +-2 mm): the matrix-product
    engines equal the per-term sum, and the separable oracle."""
    pts = scenes.pls_scene(11, 5000)
    p = PlsParams(1024, 1024, 8e-6, 8e-6, 0.0, 0.0, 0.0, 0.0, 532e-9, 0.0, 0.0, _lib.PLS_FRESNEL, 1,
                  _lib.PLS_ENGINE_DIRECT)
    direct = _run(ctx, "fp32", p, pts)
    p.engine = _lib.PLS_ENGINE_GEMM
    gemm = _run(ctx, "fp32", p, pts)
    p.engine = _lib.PLS_ENGINE_AUTO
    auto = _run(ctx, "fp32", p, pts)
    ref = opls.pls_fresnel_separable(pts[:, :].astype(np.float64), 1024, 1024, 8e-6, 8e-6, 532e-9, 0.0,
                                     use_amplitude=True)
    assert _rel(direct, ref) < TOL_F32
    assert _rel(gemm, ref) < TOL_F32
    assert _rel(auto, ref) < TOL_TENSOR


def test_pls_zero_points_and_singular_points(ctx):
    p = PlsParams(32, 16, 8e-6, 8e-6, 0.0, 0.0, 0.0, 0.0, 532e-9, 0.01, 0.0, _lib.PLS_FRESNEL, 0,
                  _lib.PLS_ENGINE_DIRECT)
    out = torch.full((16, 32), 5.0, dtype=torch.complex64, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("oh_pls", ctx.handle, 0, C.byref(p), None, 0, C.c_void_p(out.data_ptr()), st)
    torch.cuda.synchronize()
    assert torch.count_nonzero(out).item() == 0
    # a point at dz = z_k + z = 0 exactly (the reference divides by zero) contributes nothing
    pts = scenes.pls_scene(4, 20, xy_half=0.1e-3, z_range=(0.02, 0.03))
    bad = pts.copy()
    bad[5, 4] = -0.01
    p.z = -float(bad[5, 4])
    ref = _ref(p, np.delete(bad, 5, axis=0))
    got = _run(ctx, "fp32", p, bad)
    assert np.all(np.isfinite(got)) and _rel(got, ref) < TOL_F32


def test_pls_rejects_bad_arguments(ctx):
    p = PlsParams(32, 16, 8e-6, 8e-6, 0.0, 0.0, 0.0, 0.0, 532e-9, 0.01, 0.0, 7, 0, 0)
    out = torch.empty((16, 32), dtype=torch.complex64, device="cuda")
    with pytest.raises(OhError):
        _lib.call("oh_pls", ctx.handle, 0, C.byref(p), None, 0, C.c_void_p(out.data_ptr()), None)


def test_point_light_sources_class(ctx):
    pts = scenes.pls_scene(5, 200, xy_half=0.2e-3, z_range=(0.02, 0.03), amplitude=False)
    pls = PointLightSources(ctx, 64, 48, pitch=(8e-6, 8e-6), lam=633e-9)
    pls.set_points(pts)
    u = pls.Fresnel(0.005, 0.2).cpu().numpy()
    i = pls.CGHFresnel(0.005, 0.2).cpu().numpy()
    ref = opls.pls(pts, 64, 48, 8e-6, 8e-6, 633e-9, 0.005, 0.2, opls.FRESNEL)
    assert _rel(u, ref) < TOL_TENSOR
    assert _rel(i, ref.real) < TOL_TENSOR
