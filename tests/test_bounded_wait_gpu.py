"""The bounded device-side waits' error path, made to run out on purpose.

oh_ctx_set_test_stall makes the selected kernels first wait on a device flag
that nothing sets, for a short bound (about 1 ms of SM clock here), and then
take the same path as a copy or tensor-core stage that never completes: let
their copies and MMAs land, free tensor memory, set the context's error word
and return.  Each test checks that oh_ctx_device_status reports
OH_ERR_TIMEOUT, and that the next call on the same context, with the hook
off, succeeds and matches the oracle (the context stays usable)."""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, depthmap as dm, scenes
from oracle import depthmap as odm
from oracle import pls as opls
from oracle import unet as U

pytestmark = pytest.mark.gpu

STALL = 2_000_000          # SM clocks (~1 ms)
TIMEOUT = 5                # OH_ERR_TIMEOUT


def S():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def status(ctx):
    return _lib.lib().oh_ctx_device_status(ctx.handle, S())


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture
def stall(ctx):
    def on(mask):
        _lib.call("oh_ctx_set_test_stall", ctx.handle, mask, STALL)
    yield on
    _lib.call("oh_ctx_set_test_stall", ctx.handle, 0, 0)
    status(ctx)


def test_depthmap_column_pass_wait_runs_out(ctx, stall):
    ny, nx = 540, 960
    img, depth = scenes.depthmap_scene(4, ny, nx)
    p = dm.make_params(pnx=nx, pny=ny, num_of_depth=8, pad=2, phase_mode=dm.OH_PHASE_SEEDED, seed=3)
    ti, td = torch.from_numpy(img).cuda(), torch.from_numpy(depth).cuda()
    assert status(ctx) == 0
    stall(1)
    dm.generate(ctx, p, ti, td)
    assert status(ctx) == TIMEOUT
    _lib.call("oh_ctx_set_test_stall", ctx.handle, 0, 0)
    fr = dm.generate(ctx, p, ti, td)
    assert status(ctx) == 0
    op = odm.DMParams(pnx=nx, pny=ny, num_of_depth=8, pad=2)
    ref = odm.generate(img, depth, op, phase=scenes.seeded_phase(3, ny, nx))[0]
    assert rel(fr.cpu().numpy(), ref) < 1e-3


def test_point_sum_tensor_gemm_wait_runs_out(ctx, stall):
    n, nx, ny = 600, 256, 128
    pts = scenes.pls_scene(3, n)
    tp = torch.from_numpy(pts).cuda()
    out = torch.empty((ny, nx), dtype=torch.complex64, device="cuda")
    pp = _lib.PlsParams(nx, ny, 8e-6, 8e-6, 0.0, 0.0, 0.0, 0.0, 532e-9, 0.0, 0.0, _lib.PLS_FRESNEL, 1,
                        _lib.PLS_ENGINE_TENSOR)
    run = lambda: _lib.call("oh_pls", ctx.handle, 0, C.byref(pp), C.c_void_p(tp.data_ptr()), n,
                            C.c_void_p(out.data_ptr()), S())
    stall(2)
    run()
    assert status(ctx) == TIMEOUT
    _lib.call("oh_ctx_set_test_stall", ctx.handle, 0, 0)
    run()
    assert status(ctx) == 0
    ref = opls.pls(pts, nx, ny, 8e-6, 8e-6, 532e-9, 0.0, 0.0, opls.FRESNEL, use_amplitude=True)
    assert rel(out.cpu().numpy(), ref) < 1e-4


def test_convolution_waits_run_out(ctx, stall):
    rng = np.random.default_rng(1)
    n, h, w, cin, cout = 1, 8, 128, 32, 64
    x = torch.from_numpy(rng.standard_normal((n, h, w, cin)).astype(np.float32)).to(torch.bfloat16).cuda()
    W = torch.from_numpy((rng.standard_normal((cout, 9 * cin)) * 0.05).astype(np.float32)).to(torch.bfloat16).cuda()
    y = torch.zeros((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    dwt = torch.zeros((9 * cin, cout), dtype=torch.float32, device="cuda")
    P = lambda t: C.c_void_p(t.data_ptr())
    fwd = lambda: _lib.call("oh_conv2d_bf16", ctx.handle, 9, 1, n, h, w, cin, cout, P(x), cin, P(W), None, 0, None, 0,
                            P(y), cout, S())
    wg = lambda: _lib.call("oh_conv2d_wgrad_bf16", ctx.handle, 9, n, h, w, cin, cout, P(x), cin, P(y), cout, P(dwt),
                           S())
    stall(4)
    fwd()
    assert status(ctx) == TIMEOUT
    assert float(y.float().abs().max()) == 0.0          # the aborted launch wrote nothing
    wg()
    assert status(ctx) == TIMEOUT
    assert float(dwt.abs().max()) == 0.0
    _lib.call("oh_ctx_set_test_stall", ctx.handle, 0, 0)
    fwd()
    assert status(ctx) == 0
    xn = x.float().cpu().numpy().astype(np.float64)
    Wn = W.float().cpu().numpy().astype(np.float64).reshape(cout, 9, cin)
    assert rel(y.float().cpu().numpy(), U.conv(xn, Wn)) < 6e-3
