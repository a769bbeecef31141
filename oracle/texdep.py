"""CPU oracle for the texture/depth WRP of CWO++ (cwoTexDep::WRP) — TEST INFRASTRUCTURE ONLY.

Restates OpenHolo_WRP/openwrp_console_ver 1.0/cwo/src/cwoTexDep.cpp in FP64,
as the reference's per-texel scatter (AddPixel inside the plane only):

  wrp_single (cwoTexDep.cpp:29-75): every texel with tex = int(value) != 0
    adds tex exp(i k r) at (tx + wx, ty + wy) for wx, wy in [-w, w),
    r = z + ((wx px)^2 + (wy py)^2) / (2 z), w = int(|z| tan(asin(lambda / (2 px))) / px).
  wrp_range (cwoTexDep.cpp:78-136): texels with dep in [lo, hi) use
    dz = z + (hi - dep) dz_step, w = int(int(|dz| tan(asin(lambda/(2 px)))/px) / 1.4),
    wy in [-w, 0) (half zone plate), wx in [-w, w), r = (dx^2 + dy^2) / (2 dz).
    The reference sets dep from the texture value when a depth image is
    loaded (it copies the pixel into dep before reading the depth image into
    the same variable) and to 0 without one; dep_from_texture selects that
    behaviour, otherwise dep is the depth image's value.

lambda and the pitches are used as the float values the reference holds; the
phases are evaluated in double (the reference forms k r in float).  Parity
unpinned: cwoTexDep needs the CWO base class and the absent CWO++ DLL.
"""
from __future__ import annotations

import numpy as np


def _f32(v):
    return float(np.float32(v))


def half_width(dz, lam, px):
    lam, px = _f32(lam), _f32(px)
    return int(abs(dz) * np.tan(np.arcsin(lam / (2.0 * px))) / px)


def _scatter(out, tx, ty, val, wxs, wys, ph):
    ny, nx = out.shape
    for a, wy in enumerate(wys):
        y = ty + wy
        if y < 0 or y >= ny:
            continue
        xs = tx + wxs
        ok = (xs >= 0) & (xs < nx)
        out[y, xs[ok]] += val * np.exp(1j * ph[a, ok])


def wrp_single(tex, px, py, lam, z):
    tex = np.asarray(tex)
    ny, nx = tex.shape
    k = 2 * np.pi / _f32(lam)
    px, py = _f32(px), _f32(py)
    w = half_width(z, lam, px)
    out = np.zeros((ny, nx), np.complex128)
    if w <= 0:
        return out
    wxs = np.arange(-w, w)
    wys = np.arange(-w, w)
    r = z + ((wxs[None, :] * px) ** 2 + (wys[:, None] * py) ** 2) / (2.0 * z)
    ph = k * r
    for ty in range(ny):
        for tx in range(nx):
            t = int(tex[ty, tx])
            if t != 0:
                _scatter(out, tx, ty, t, wxs, wys, ph)
    return out


def wrp_range(tex, dep, px, py, lam, z, dz_step, lo, hi, dep_from_texture=True):
    tex = np.asarray(tex)
    ny, nx = tex.shape
    k = 2 * np.pi / _f32(lam)
    px, py = _f32(px), _f32(py)
    out = np.zeros((ny, nx), np.complex128)
    for ty in range(ny):
        for tx in range(nx):
            t = int(tex[ty, tx])
            if t == 0:
                continue
            if dep is None:
                d = 0
            else:
                d = t if dep_from_texture else int(dep[ty, tx])
            if not (lo <= d < hi):
                continue
            dz = z + (hi - d) * dz_step
            w = int(half_width(dz, lam, px) / 1.4)
            if w <= 0:
                continue
            wxs = np.arange(-w, w)
            wys = np.arange(-w, 0)
            ph = k * ((wxs[None, :] * px) ** 2 + (wys[:, None] * py) ** 2) / (2.0 * dz)
            _scatter(out, tx, ty, t, wxs, wys, ph)
    return out
