"""oh_reconstruct_eye (HologramGenerator::ReconstructImage, one frame) against
the FP64 restatement, on random fringes and on a depth-map hologram of this
library, with the reference's shift convention at odd sizes and its
test_pixel_number_scale."""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, depthmap as dm, scenes
from openholo_gb300._lib import EyeParams, OhError
from oracle import reconstruct as orec

pytestmark = pytest.mark.gpu


def _run(ctx, prec, p, fringe):
    dt = torch.float64 if prec == "fp64" else torch.float32
    f = torch.as_tensor(fringe).to(dt).cuda().contiguous()
    out = torch.empty((p.pny // p.pixel_scale, p.pnx // p.pixel_scale), dtype=dt, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("oh_reconstruct_eye", ctx.handle, 1 if prec == "fp64" else 0, C.byref(p), C.c_void_p(f.data_ptr()),
              C.c_void_p(out.data_ptr()), st)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _ref(p, fringe):
    return orec.reconstruct_eye(fringe, p.pnx, p.pny, p.ppx, p.ppy, p.lambda_, p.field_lens, p.eye_length,
                                p.eye_pupil_diameter, p.eye_center_x, p.eye_center_y, p.focus_distance,
                                p.pixel_scale)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _signal(p, ref, fringe):
    # the eye's apertures must pass a real part of the light, or the
    # comparison would be between rounding residues
    assert np.linalg.norm(ref) > 1e-3 * np.linalg.norm(fringe)


# SLM apertures of a few mm (pitch 100 um) so that the eye lens' anti-aliasing
# radius, about (f - d) N p / (2 f), spans many eye-plane pixels
@pytest.mark.parametrize("shape,scale,center,focus", [((48, 64), 1, (0.0, 1e-3), 0.5),
                                                     ((45, 63), 1, (-2e-3, 3e-3), 0.45),
                                                     ((64, 96), 2, (0.0, 0.0), 0.6)])
def test_random_fringe(ctx, shape, scale, center, focus):
    ny, nx = shape
    fringe = np.random.default_rng(7).random((ny, nx))
    p = EyeParams(nx, ny, 100e-6, 100e-6, 532e-9, 1.0, scale, 50e-3, 6e-3, center[0], center[1], focus)
    ref = _ref(p, fringe)
    _signal(p, ref, fringe)
    assert _rel(_run(ctx, "fp64", p, fringe), ref) < 1e-10
    assert _rel(_run(ctx, "fp32", p, fringe), ref) < 1e-5


def test_depthmap_hologram_focus_sweep(ctx):
    ny, nx = 108, 192
    img, depth = scenes.depthmap_scene(3, ny, nx)
    pp = dm.make_params(pnx=nx, pny=ny, ppx=50e-6, ppy=50e-6, num_of_depth=8, near=0.3, far=0.35, pad=1)
    fr = dm.generate(ctx, pp, torch.from_numpy(img).cuda(), torch.from_numpy(depth).cuda(), precision="fp64")
    torch.cuda.synchronize()
    fringe = fr.cpu().numpy()
    for focus in (0.30, 0.325, 0.35):
        p = EyeParams(nx, ny, 50e-6, 50e-6, 532e-9, 1.0, 1, 50e-3, 6e-3, 0.0, 0.0, focus)
        ref = _ref(p, fringe)
        _signal(p, ref, fringe)
        assert _rel(_run(ctx, "fp64", p, fringe), ref) < 1e-10
        assert _rel(_run(ctx, "fp32", p, fringe), ref) < 1e-5


def test_rejects_focus_at_field_lens(ctx):
    p = EyeParams(16, 16, 8e-6, 8e-6, 532e-9, 1.0, 1, 50e-3, 6e-3, 0.0, 0.0, 1.0)
    f = torch.zeros((16, 16), dtype=torch.float32, device="cuda")
    with pytest.raises(OhError):
        _lib.call("oh_reconstruct_eye", ctx.handle, 0, C.byref(p), C.c_void_p(f.data_ptr()),
                  C.c_void_p(f.data_ptr()), None)
