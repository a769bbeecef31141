"""The library's mixed-radix FFT against numpy (pocketfft, float64)."""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib
from openholo_gb300._lib import OhError

pytestmark = pytest.mark.gpu


def fft2(ctx, x, direction=-1, shift=0, normalize=0, precision="fp64", inplace=False):
    dt = torch.complex128 if precision == "fp64" else torch.complex64
    t = torch.from_numpy(x.astype(np.complex128)).to(dt).cuda()
    out = t if inplace else torch.empty_like(t)
    ny, nx = x.shape
    _lib.call("oh_fft2d", ctx.handle, 1 if precision == "fp64" else 0, nx, ny, C.c_void_p(t.data_ptr()),
              C.c_void_p(out.data_ptr()), direction, shift, normalize,
              C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return out.cpu().numpy()


SIZES = [(1, 1), (1, 8), (8, 1), (16, 16), (6, 10), (30, 64), (27, 125), (49, 14), (81, 32), (11, 13),
         (120, 90), (2160, 8), (8, 3840), (1080, 16), (48, 1920), (12, 59)]


@pytest.mark.parametrize("shape", SIZES)
def test_fft2_forward_inverse(ctx, shape):
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    ref = np.fft.fft2(x)
    got = fft2(ctx, x, -1)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref) * np.log2(max(x.size, 2))
    got32 = fft2(ctx, x, -1, precision="fp32")
    assert np.linalg.norm(got32 - ref) <= 1e-6 * np.linalg.norm(ref) * np.log2(max(x.size, 2))
    back = fft2(ctx, ref, +1, normalize=1)
    assert np.linalg.norm(back - x) <= 1e-12 * np.linalg.norm(x) * np.log2(max(x.size, 2))


@pytest.mark.parametrize("shape", [(6, 8), (7, 9), (1080, 1920)])
def test_fft2_shifted(ctx, shape):
    rng = np.random.default_rng(3)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    ref = np.fft.fftshift(np.fft.fft2(np.fft.fftshift(x)))
    got = fft2(ctx, x, -1, shift=1)
    assert np.linalg.norm(got - ref) <= 1e-11 * np.linalg.norm(ref)
    ref_inv = np.fft.fftshift(np.fft.ifft2(np.fft.fftshift(x)))
    got_inv = fft2(ctx, x, +1, shift=1, normalize=1)
    assert np.linalg.norm(got_inv - ref_inv) <= 1e-11 * np.linalg.norm(ref_inv)


def test_fft2_in_place(ctx):
    x = np.random.default_rng(9).standard_normal((36, 40)) + 0j
    got = fft2(ctx, x, -1, shift=1, inplace=True)
    assert np.allclose(got, np.fft.fftshift(np.fft.fft2(np.fft.fftshift(x))), atol=1e-10)


def test_fft1d_rows(ctx):
    x = np.random.default_rng(4).standard_normal((5, 3840)) + 1j
    t = torch.from_numpy(x).cuda()
    out = torch.empty_like(t)
    _lib.call("oh_fft1d_rows", ctx.handle, 1, 3840, 5, C.c_void_p(t.data_ptr()), C.c_void_p(out.data_ptr()), -1, 0,
              C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    ref = np.fft.fft(x, axis=1)
    assert np.linalg.norm(out.cpu().numpy() - ref) <= 1e-12 * np.linalg.norm(ref) * 12


def test_fft_supported_and_errors(ctx):
    L = _lib.lib()
    assert L.oh_fft_supported(3840, 0) == 1 and L.oh_fft_supported(2160, 1) == 1
    assert L.oh_fft_supported(67, 0) == 0          # prime above the generic radix limit
    assert L.oh_fft_supported(0, 0) == 0
    x = np.ones((4, 67), np.complex128)
    with pytest.raises(OhError):
        fft2(ctx, x)
    with pytest.raises(OhError):
        fft2(ctx, np.ones((4, 4)), direction=0)


@pytest.mark.parametrize("shape", [(120, 90), (1080, 1920), (27, 125)])
def test_fft2_parseval(ctx, shape):
    # known answer: the unnormalised forward transform multiplies the energy by N
    rng = np.random.default_rng(7)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    for precision, tol in (("fp64", 1e-12), ("fp32", 1e-6)):
        X = fft2(ctx, x, -1, precision=precision)
        ex, eX = np.sum(np.abs(x) ** 2), np.sum(np.abs(X) ** 2) / x.size
        assert abs(eX - ex) <= tol * ex, precision
