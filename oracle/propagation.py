"""CPU oracle for the MATLAB tools' propagation forms — TEST INFRASTRUCTURE ONLY.

as_bandlimited restates fn_FresnelPropagation_as.m:1-48 (OpenHolo_MeshCGH)
in numpy, step for step with its 1-based indices translated to 0-based:
2x zero pad with the input at rows/columns round(N/2)-1 .., centred FFT
(fftshift(fft2(ifftshift(.)))), kernel exp(i 2 pi z sqrt(1/lambda^2 - a^2 - b^2))
on the MATLAB grid a = ((1:2Nx) - Nx) da (a one-sample offset from the FFT
grid, kept), the Matsushima band limit with sx = sy = 0, centred inverse FFT,
crop.  MATLAB's sqrt of a negative number is imaginary, which makes the
evanescent kernel exp(-2 pi z sqrt(|q|)); numpy's complex sqrt does the same.
fresnel_tf (FresnelPropagation.m) lives in oracle/wrp.py.  No reference
output pins either (MATLAB is not available): parity unpinned.
"""
from __future__ import annotations

import math

import numpy as np


def _matlab_round_half(n: int) -> int:
    """round(n / 2) for a positive integer n (MATLAB rounds halves away from zero)."""
    return int(math.floor(n / 2 + 0.5))


def as_bandlimited(inp, dx, dy, z, lam):
    inp = np.asarray(inp, dtype=np.complex128)
    ny, nx = inp.shape
    nxx, nyy = 2 * nx, 2 * ny
    pad = np.zeros((nyy, nxx), np.complex128)
    sx = _matlab_round_half(nx) - 1
    sy = _matlab_round_half(ny) - 1
    pad[sy:sy + ny, sx:sx + nx] = inp
    dal = 1.0 / (nxx * dx)
    dbl = 1.0 / (nyy * dy)
    al, bl = np.meshgrid((np.arange(1, nxx + 1) - nxx / 2) * dal, (np.arange(1, nyy + 1) - nyy / 2) * dbl)
    A = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(pad)))
    sq = np.sqrt((1.0 / lam ** 2 - al ** 2 - bl ** 2).astype(np.complex128))
    kern = np.exp(1j * 2 * np.pi * z * sq)
    with np.errstate(divide="ignore", invalid="ignore"):
        fla = np.abs(-al * z / sq)
        flb = np.abs(-bl * z / sq)
    kern[fla > 1.0 / (2 * dal)] = 0
    kern[flb > 1.0 / (2 * dbl)] = 0
    inter = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(A * kern)))
    return inter[sy:sy + ny, sx:sx + nx]
