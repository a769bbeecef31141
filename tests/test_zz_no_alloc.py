"""oh_pointcloud_noalloc: the allocation-free point-cloud entry point.

Some callers cannot allocate device memory once running (an SLM/display loop
under a fixed memory budget, or a host framework that owns all device
allocations).  This entry point takes no context and keeps its working tables
in a fixed device array inside the library.  It must give the same field and
fringe as the regular entry point (oh_pointcloud, which uses the context's
scratch), call after call.  This file is collected last so that a failure
here does not hide the other tests; it also passes when run on its own.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, scenes
from openholo_gb300._lib import OhError, PcParams

pytestmark = pytest.mark.gpu

TOL = 1e-5   # FP32: chunk boundaries differ between the two entry points (summation order)


def _params(nx, ny, tilt=(0.0, 0.0)):
    return PcParams(1.0, 1.0, 1.0, 0.0, 8e-6, 8e-6, nx, ny, 532e-9, tilt[0], tilt[1])


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _regular(ctx, p, pts):
    field = torch.empty((p.ny, p.nx), dtype=torch.complex64, device="cuda")
    fringe = torch.zeros((p.ny, p.nx), dtype=torch.float32, device="cuda")
    _lib.call("oh_pointcloud", ctx.handle, 0, C.byref(p), C.c_void_p(pts.data_ptr()), pts.shape[0],
              C.c_void_p(field.data_ptr()), C.c_void_p(fringe.data_ptr()), _stream())
    return field, fringe


def _noalloc(p, pts):
    field = torch.empty((p.ny, p.nx), dtype=torch.complex64, device="cuda")
    fringe = torch.zeros((p.ny, p.nx), dtype=torch.float32, device="cuda")
    _lib.call("oh_pointcloud_noalloc", C.byref(p), C.c_void_p(pts.data_ptr()), pts.shape[0],
              C.c_void_p(field.data_ptr()), C.c_void_p(fringe.data_ptr()), _stream())
    return field, fringe


def _rel(a, b):
    wide = torch.complex128 if a.is_complex() else torch.float64
    a, b = a.to(wide), b.to(wide)
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


@pytest.mark.parametrize("shape,n", [((256, 320), 3000), ((1024, 1024), 900)])
def test_noalloc_matches_regular_entry_point(ctx, shape, n):
    ny, nx = shape
    p = _params(nx, ny, tilt=(3.0, -2.0))
    pts = torch.from_numpy(scenes.pointcloud_scene(5, n).astype(np.float32)).cuda()
    ref_field, ref_fringe = _regular(ctx, p, pts)
    for _ in range(2):                       # two calls in a row share the fixed scratch
        field, fringe = _noalloc(p, pts)
        torch.cuda.synchronize()
        assert _rel(field, ref_field) < TOL
        assert _rel(fringe, ref_fringe) < TOL


def test_noalloc_leaves_device_memory_unchanged(ctx):
    """After a first call (which looks up the array's address), a call takes
    no device memory: the device's free bytes and torch's allocations are
    the same before and after it, and its result still equals the regular
    entry point's."""
    p = _params(512, 384)
    pts = torch.from_numpy(scenes.pointcloud_scene(8, 2000).astype(np.float32)).cuda()
    ref_field, _ = _regular(ctx, p, pts)
    field = torch.empty((p.ny, p.nx), dtype=torch.complex64, device="cuda")
    call = lambda: _lib.call("oh_pointcloud_noalloc", C.byref(p), C.c_void_p(pts.data_ptr()), pts.shape[0],
                             C.c_void_p(field.data_ptr()), None, _stream())
    call()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    torch_bytes0 = torch.cuda.memory_allocated()
    field.zero_()
    torch.cuda.synchronize()
    call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == torch_bytes0
    assert _rel(field, ref_field) < TOL


def test_noalloc_rejects_fields_beyond_its_scratch(lib_built):
    p = _params(16384, 16384)
    pts = torch.zeros((4, 4), dtype=torch.float32, device="cuda")
    out = torch.empty((1, 1), dtype=torch.complex64, device="cuda")
    with pytest.raises(OhError) as ei:
        _lib.call("oh_pointcloud_noalloc", C.byref(p), C.c_void_p(pts.data_ptr()), 4, C.c_void_p(out.data_ptr()), None,
                  _stream())
    assert "2*nx + 3*ny" in str(ei.value)
