"""oh_mesh_hologram (MeshCGH: fn_genH with flat or continuous shading)
against the FP64 restatement."""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, scenes
from openholo_gb300._lib import MeshParams, OhError
from oracle import mesh as omesh

pytestmark = pytest.mark.gpu

TOL = 1e-8    # both sides reduce phases of ~1e5 turns in double (~1e-10 rad each)


def _run(ctx, p, tris, spectrum=False):
    field = torch.empty((p.ny, p.nx), dtype=torch.complex128, device="cuda")
    spec = torch.empty_like(field) if spectrum else None
    t = np.ascontiguousarray(tris, np.float64)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("oh_mesh_hologram", ctx.handle, C.byref(p), t.ctypes.data_as(C.c_void_p), t.shape[0],
              C.c_void_p(field.data_ptr()), C.c_void_p(spec.data_ptr()) if spec is not None else None, st)
    torch.cuda.synchronize()
    return (field.cpu().numpy(), spec.cpu().numpy()) if spectrum else field.cpu().numpy()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("continuous", [0, 1])
@pytest.mark.parametrize("shape", [(48, 64), (33, 40)])
def test_mesh_matches_oracle(ctx, continuous, shape):
    ny, nx = shape
    tris = scenes.mesh_scene(5, cells=4, size=nx * 8e-6 / 3)
    illu = (1.0, 1.0, 1.0)
    p = MeshParams(nx, ny, 8e-6, 8e-6, 532e-9, (C.c_double * 3)(*illu), continuous)
    got, spec = _run(ctx, p, tris, spectrum=True)
    ref, ref_spec = omesh.gen_hologram(tris, nx, ny, 8e-6, 8e-6, 532e-9, illu, bool(continuous), return_spectrum=True)
    assert np.linalg.norm(ref) > 0
    # near the reference triangle's removable singularities the source's
    # formulas cancel (order 1/f flat, 1/f^2 continuous): compare tightly
    # elsewhere, and bound the whole field
    bad = omesh.ill_conditioned(tris, nx, ny, 8e-6, 8e-6, 532e-9, bool(continuous))
    assert bad.mean() < 0.2
    good = ~bad
    assert _rel(spec[good], ref_spec[good]) < TOL
    assert _rel(spec, ref_spec) < (TOL if not continuous else 1e-3)
    assert _rel(got, ref) < (TOL if not continuous else 1e-3)


def test_mesh_no_visible_triangles_and_bad_pitch(ctx):
    tris = scenes.mesh_scene(2, cells=1, back_facing=0)[:2]
    flipped = tris.reshape(-1, 3, 3)[:, [0, 2, 1]].reshape(-1, 9)
    p = MeshParams(16, 16, 8e-6, 8e-6, 532e-9, (C.c_double * 3)(0.0, 0.0, 0.0), 0)
    assert np.count_nonzero(_run(ctx, p, flipped)) == 0
    p.dx = 0.4e-6                 # below the wavelength
    with pytest.raises(OhError):
        _run(ctx, p, tris)
