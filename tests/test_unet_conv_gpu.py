"""Tensor-core implicit-GEMM convolutions (oh_conv2d_bf16 forward and input
gradient, oh_conv2d_wgrad_bf16) against the float64 oracle on the same BF16
inputs.  The products are exact in FP32 and accumulate in FP32; the forward
and input-gradient outputs are rounded to BF16 (relative 2^-9), so the bound
is 6e-3 relative L2 for those and 1e-4 for the FP32 weight gradient."""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib
from oracle import unet as U

pytestmark = pytest.mark.gpu


def S():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def P(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def bf16(rng, shape, scale=1.0):
    return torch.from_numpy((rng.standard_normal(shape) * scale).astype(np.float32)).to(torch.bfloat16).cuda()


@pytest.mark.parametrize("n,h,w,cin,cout,taps", [(1, 16, 128, 32, 32, 9), (2, 12, 32, 64, 128, 9),
                                                 (1, 9, 200, 96, 64, 9), (1, 8, 256, 256, 256, 9),
                                                 (2, 4, 8, 64, 384, 9), (1, 16, 128, 64, 32, 1)])
def test_conv_forward(ctx, n, h, w, cin, cout, taps):
    rng = np.random.default_rng(n * 1000 + cin + cout + w)
    xs = cin + 32                               # a channel stride wider than cin
    x = bf16(rng, (n, h, w, xs))
    W = bf16(rng, (cout, taps * cin), (2.0 / (taps * cin)) ** 0.5)
    b = torch.from_numpy(rng.standard_normal(cout).astype(np.float32) * 0.1).cuda()
    os_ = cout + 32                             # output written into a wider buffer
    out = torch.full((n, h, w, os_), 7.0, dtype=torch.bfloat16, device="cuda")
    _lib.call("oh_conv2d_bf16", ctx.handle, taps, 1, n, h, w, cin, cout, P(x), xs, P(W), P(b), 1, None, 0, P(out),
              os_, S())
    torch.cuda.synchronize()
    xn = x.float().cpu().numpy()[..., :cin].astype(np.float64)
    Wn = W.float().cpu().numpy().astype(np.float64).reshape(cout, taps, cin)
    ref = U.conv(xn, Wn, b.cpu().numpy().astype(np.float64), relu=True)
    got = out.float().cpu().numpy()
    assert rel(got[..., :cout], ref) < 6e-3
    assert np.all(got[..., cout:] == 7.0)      # channels past cout untouched


@pytest.mark.parametrize("n,h,w,cin,cout", [(1, 16, 128, 32, 64), (2, 8, 64, 96, 32), (1, 6, 160, 64, 128)])
def test_conv_input_gradient_with_mask(ctx, n, h, w, cin, cout):
    """sign = -1 with the transposed weights, times the ReLU mask of the
    layer input: the input gradient of a 3x3 layer."""
    rng = np.random.default_rng(cin * 7 + cout)
    dz = bf16(rng, (n, h, w, cout))
    W = rng.standard_normal((cout, 9, cin)) * (2.0 / (9 * cin)) ** 0.5
    Wt = torch.from_numpy(np.ascontiguousarray(np.transpose(W, (2, 1, 0)).reshape(cin, 9 * cout)).astype(
        np.float32)).to(torch.bfloat16).cuda()
    mask = bf16(rng, (n, h, w, cin))
    out = torch.empty((n, h, w, cin), dtype=torch.bfloat16, device="cuda")
    _lib.call("oh_conv2d_bf16", ctx.handle, 9, -1, n, h, w, cout, cin, P(dz), cout, P(Wt), None, 0, P(mask), cin,
              P(out), cin, S())
    torch.cuda.synchronize()
    Wq = Wt.float().cpu().numpy().astype(np.float64).reshape(cin, 9, cout).transpose(2, 1, 0)
    ref = U.conv_dgrad(dz.float().cpu().numpy().astype(np.float64), Wq) * (mask.float().cpu().numpy() > 0)
    assert rel(out.float().cpu().numpy(), ref) < 6e-3


@pytest.mark.parametrize("n,h,w,cin,cout,taps", [(1, 16, 128, 32, 32, 9), (2, 12, 64, 96, 64, 9),
                                                 (1, 8, 16, 64, 128, 9), (1, 32, 96, 128, 256, 9),
                                                 (1, 8, 128, 32, 64, 1), (1, 8, 128, 64, 128, 9),
                                                 (2, 6, 100, 32, 32, 9), (1, 4, 192, 192, 64, 9)])
def test_conv_weight_gradient(ctx, n, h, w, cin, cout, taps):
    """Widths of at least 64 with 3x3 taps and up to 128 output channels run
    the row-box kernel (three dx taps from one load); the others the
    four-group kernel."""
    rng = np.random.default_rng(cin + cout + h)
    x = bf16(rng, (n, h, w, cin))
    dz = bf16(rng, (n, h, w, cout))
    dwt = torch.zeros((taps * cin, cout), dtype=torch.float32, device="cuda")
    for _ in range(2):                         # accumulates: two calls give twice the gradient
        _lib.call("oh_conv2d_wgrad_bf16", ctx.handle, taps, n, h, w, cin, cout, P(x), cin, P(dz), cout, P(dwt), S())
    torch.cuda.synchronize()
    ref = U.conv_wgrad(x.float().cpu().numpy().astype(np.float64), dz.float().cpu().numpy().astype(np.float64), taps)
    ref_t = 2.0 * np.transpose(ref, (1, 2, 0)).reshape(taps * cin, cout)
    assert rel(dwt.cpu().numpy(), ref_t) < 1e-4


def test_conv_rejects_bad_shapes(ctx):
    x = torch.zeros((1, 4, 48, 32), dtype=torch.bfloat16, device="cuda")
    W = torch.zeros((32, 288), dtype=torch.bfloat16, device="cuda")
    with pytest.raises(_lib.OhError):          # width 48 does not divide 128
        _lib.call("oh_conv2d_bf16", ctx.handle, 9, 1, 1, 4, 48, 32, 32, P(x), 32, P(W), None, 0, None, 0, P(x), 32, S())
    with pytest.raises(_lib.OhError):          # cin not a multiple of 32
        _lib.call("oh_conv2d_bf16", ctx.handle, 9, 1, 1, 4, 32, 16, 32, P(x), 32, P(W), None, 0, None, 0, P(x), 32, S())
