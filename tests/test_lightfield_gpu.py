"""oh_lightfield_to_field (LF-CGH) against the numpy restatement."""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, scenes
from oracle import lightfield as olf

pytestmark = pytest.mark.gpu


def _run(ctx, prec, lf, phase, seed=0):
    nt, ns, nv, nu = lf.shape
    cdt = torch.complex128 if prec == "fp64" else torch.complex64
    out = torch.empty((nt * nv, ns * nu), dtype=cdt, device="cuda")
    tl = torch.from_numpy(np.ascontiguousarray(lf, np.float32)).cuda()
    tp = torch.from_numpy(np.ascontiguousarray(phase, np.float32)).cuda() if phase is not None else None
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("oh_lightfield_to_field", ctx.handle, 1 if prec == "fp64" else 0, nu, nv, ns, nt,
              C.c_void_p(tl.data_ptr()), C.c_void_p(tp.data_ptr()) if tp is not None else None, seed,
              C.c_void_p(out.data_ptr()), st)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("shape", [(2, 3, 32, 48), (3, 2, 15, 21), (4, 4, 64, 64)])
def test_explicit_phase(ctx, shape):
    rng = np.random.default_rng(2)
    lf = rng.random(shape).astype(np.float32)
    phase = (rng.random(shape) * 2 * np.pi).astype(np.float32)
    ref = olf.lightfield_to_field(lf, phase)
    assert _rel(_run(ctx, "fp64", lf, phase), ref) < 1e-10
    assert _rel(_run(ctx, "fp32", lf, phase), ref) < 1e-5


def test_seeded_phase(ctx):
    shape = (2, 2, 24, 40)
    lf = np.random.default_rng(3).random(shape).astype(np.float32)
    seed = 12345
    phase = (2 * np.pi * scenes.u24(seed, lf.size).astype(np.float64)).reshape(shape)
    ref = olf.lightfield_to_field(lf, phase)
    assert _rel(_run(ctx, "fp64", lf, None, seed), ref) < 1e-7
