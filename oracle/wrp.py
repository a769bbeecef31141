"""CPU oracle for Fresnel propagation — TEST INFRASTRUCTURE ONLY.

fresnel_conv: CWO::Diffract(z, CWO_FRESNEL_CONV) structure (WRPC/cwo/src/
cwo.cpp:2198-2279 zero-pad expand at offset N/2, DiffractConv FRESNEL_CONV
:2872-2898 FFT * FFT(kernel) -> IFFT -> 1/N, crop), with the impulse response
written from the mathematics (the DLL bodies are not in the tree):
h = exp(ikz)/(i lambda z) exp(i pi (x^2+y^2)/(lambda z)) dp^2, origin at
index 0.  Parity unpinned.
fresnel_tf: the transfer-function form of FresnelPropagation.m:1-16.
"""
from __future__ import annotations

import numpy as np


def fresnel_conv(U, dp, lam, z):
    ny, nx = U.shape
    NX, NY = 2 * nx, 2 * ny
    a = np.zeros((NY, NX), np.complex128)
    a[ny // 2:ny // 2 + ny, nx // 2:nx // 2 + nx] = U
    jx = np.where(np.arange(NX) < NX // 2, np.arange(NX), np.arange(NX) - NX)
    jy = np.where(np.arange(NY) < NY // 2, np.arange(NY), np.arange(NY) - NY)
    x = jx * dp
    y = jy * dp
    k = 2 * np.pi / lam
    h = np.exp(1j * k * z) / (1j * lam * z) * np.exp(1j * np.pi * (x[None, :] ** 2 + y[:, None] ** 2) / (lam * z)) * dp * dp
    out = np.fft.ifft2(np.fft.fft2(a) * np.fft.fft2(h))
    return out[ny // 2:ny // 2 + ny, nx // 2:nx // 2 + nx]


def fresnel_tf(field, dx, dy, z, lam):
    k = 2 * np.pi / lam
    ny, nx = field.shape
    fx = 1.0 / (nx * dx)
    fy = 1.0 / (ny * dy)
    xi = np.concatenate([np.arange(0, (nx - 1) // 2 + 1), np.arange(-((nx + 2) // 2) + 1, 0)]) * fx
    yi = np.concatenate([np.arange(0, (ny - 1) // 2 + 1), np.arange(-((ny + 2) // 2) + 1, 0)]) * fy
    H = np.exp(1j * k * z) * np.exp(-1j * np.pi * lam * z * (xi[None, :] ** 2 + yi[:, None] ** 2))
    return np.fft.ifft2(np.fft.fft2(field) * H)


def _mround(x):
    """MATLAB round: halves away from zero."""
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def fn_wrp_window(obj, lam, dp, res, z_wrp, phase=None):
    """fn_wrp.m:13-36 (WRP_matlab_ver 1.0): the sub-hologram loop, with the
    per-point random phase given explicitly (phase[k] radians, MATLAB draws
    rand*2*pi).  obj: (n, 3) x, y, z.  Returns the res x res complex WRP,
    first index following x as in the MATLAB source.  The padded `temp` array
    of the source is reproduced; sub-holograms that MATLAB could not place
    (negative indices) are clipped to the plane instead."""
    obj = np.asarray(obj, dtype=np.float64)
    k = 2 * np.pi / lam
    z = z_wrp - obj[:, 2]
    N = (_mround(np.abs(lam * z / dp ** 2 / 2) + 0.5) * 2 - 1).astype(np.int64)
    cx = _mround(obj[:, 0] / dp).astype(np.int64) + (res - 1) // 2      # 1-based MATLAB index
    cy = _mround(obj[:, 1] / dp).astype(np.int64) + (res - 1) // 2
    holo = np.zeros((res, res), np.complex128)
    for o in range(obj.shape[0]):
        n = int(N[o])
        t = (np.arange(n) - (n - 1) / 2) * dp
        x_run, y_run = np.meshgrid(t, t, indexing="ij")             # rows follow x
        r = np.sign(z[o]) * np.sqrt(z[o] ** 2 + y_run ** 2 + x_run ** 2)
        ph = 0.0 if phase is None else phase[o]
        sub = np.exp(1j * ph) * np.exp(1j * k * r) / r
        # hologram row i (0-based) takes sub row a = i + (n + 1) / 2 - cx
        a0 = (n + 1) // 2 - cx[o]
        b0 = (n + 1) // 2 - cy[o]
        for i in range(res):
            a = i + a0
            if a < 0 or a >= n:
                continue
            jb = np.arange(res)
            b = jb + b0
            ok = (b >= 0) & (b < n)
            holo[i, jb[ok]] += sub[a, b[ok]]
    return holo
