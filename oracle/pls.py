"""CPU oracle for point-light-source summation (cwoPLS) — TEST INFRASTRUCTURE ONLY.

Restates, in FP64 numpy, the three per-pixel sums of the CWO++ point-light-
source class (OpenHolo_WRP/openwrp_console_ver 1.0/cwo/src/cwoPLS.cpp):

  Huygens    (cwoPLS.cpp:316-368)  U[i,j] = sum_k exp(i (k r + ph)) / r,
             r = sqrt(dx^2 + dy^2 + dz^2)
  Fresnel    (cwoPLS.cpp:370-424)  U[i,j] = sum_k exp(i (k (dx^2 + dy^2) / (2 dz) + ph))
  CGHFresnel (cwoPLS.cpp:472-520)  I[i,j] = sum_k cos(k (dx^2 + dy^2) / (2 dz) + ph)

with dx = (j - Nx/2) dpx + dox - (x_k + sox), dy = (i - Ny/2) dpy + doy -
(y_k + soy), dz = z_k + z (Nx/2 = Nx >> 1).  The reference ignores the point
amplitude (the line reading it is commented out); use_amplitude=True
multiplies each term by the point's complex amplitude a_k instead.  The
reference evaluates in float (Huygens: r and the phase in double) with the
wave number rounded to float; this oracle uses double throughout.
Parity unpinned: cwoPLS needs the CWO base class and the absent CWO++ DLL, so
it cannot be built here.
"""
from __future__ import annotations

import numpy as np

HUYGENS, FRESNEL, CGH_FRESNEL = 0, 1, 2


def pls(points, nx, ny, dpx, dpy, lam, z, ph=0.0, mode=FRESNEL, dox=0.0, doy=0.0, sox=0.0, soy=0.0,
        use_amplitude=False, chunk=256):
    """points: (n, 5) array of cwoObjPoint fields (a_re, a_im, x, y, z)."""
    pts = np.asarray(points, dtype=np.float64)
    k = 2.0 * np.pi / lam
    X = (np.arange(nx) - (nx >> 1)) * dpx + dox
    Y = (np.arange(ny) - (ny >> 1)) * dpy + doy
    out = np.zeros((ny, nx), np.complex128)
    for c0 in range(0, pts.shape[0], chunk):
        p = pts[c0:c0 + chunk]
        dx = X[None, None, :] - (p[:, 2] + sox)[:, None, None]
        dy = Y[None, :, None] - (p[:, 3] + soy)[:, None, None]
        dz = (p[:, 4] + z)[:, None, None]
        if mode == HUYGENS:
            r = np.sqrt(dx * dx + dy * dy + dz * dz)
            t = np.exp(1j * (k * r + ph)) / r
        else:
            t = np.exp(1j * (k * (dx * dx + dy * dy) / (2.0 * dz) + ph))
        if use_amplitude:
            t = t * (p[:, 0] + 1j * p[:, 1])[:, None, None]
        out += t.sum(axis=0)
    return out.real.copy() if mode == CGH_FRESNEL else out


def pls_fresnel_separable(points, nx, ny, dpx, dpy, lam, z, ph=0.0, dox=0.0, doy=0.0, sox=0.0, soy=0.0,
                          use_amplitude=False):
    """The Fresnel sum as the product of its x and y factors,
    U = e^{i ph} Ey^T diag(a) Ex: the same numbers as pls(mode=FRESNEL) in
    O((nx + ny) n + nx ny n) complex multiply-adds (used at large sizes)."""
    pts = np.asarray(points, dtype=np.float64)
    k = 2.0 * np.pi / lam
    X = (np.arange(nx) - (nx >> 1)) * dpx + dox
    Y = (np.arange(ny) - (ny >> 1)) * dpy + doy
    dz = pts[:, 4] + z
    ex = np.exp(1j * k * (X[None, :] - (pts[:, 2] + sox)[:, None]) ** 2 / (2.0 * dz[:, None]))
    ey = np.exp(1j * k * (Y[None, :] - (pts[:, 3] + soy)[:, None]) ** 2 / (2.0 * dz[:, None]))
    if use_amplitude:
        ey = ey * (pts[:, 0] + 1j * pts[:, 1])[:, None]
    return np.exp(1j * ph) * (ey.T @ ex)
