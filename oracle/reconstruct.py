"""CPU oracle for the eye-model reconstruction — TEST INFRASTRUCTURE ONLY.

Restates HologramGenerator::ReconstructImage for one frame in numpy FP64,
following HologramGenerator_CPU.cpp:414-614 line by line:
Test_Propagation_to_Eye_Pupil (:486-538), Reconstruction (:543-614) with
its circshift (:663-680) and the CPU fftwShift/fftShift (:285-345), whose
shift is out[(i - n/2) mod n] = in[i] per axis (numpy's ifftshift).  The
reference's host path needs FFTW and Qt, which are absent, so parity is
unpinned.
"""
from __future__ import annotations

import math

import numpy as np


def _s(a):
    return np.fft.ifftshift(a)                 # out[(i - n//2) mod n] = in[i]


def _fftw_shift(a):
    return _s(np.fft.fft2(_s(a)))


def _circshift(a, sx, sy):
    return np.roll(np.roll(a, sx, axis=1), sy, axis=0)


def reconstruct_eye(fringe, pnx, pny, ppx, ppy, lam, field_lens, eye_length, pupil, cx, cy, focus, scale=1):
    nx, ny = pnx // scale, pny // scale
    ppx, ppy = ppx / scale, ppy / scale
    flat = np.asarray(fringe, dtype=np.float64).reshape(-1)[:nx * ny]
    hh = flat.reshape(ny, nx).astype(np.complex128)
    hh = _fftw_shift(hh)
    pp_ex, pp_ey = lam * field_lens / (nx * ppx), lam * field_lens / (ny * ppy)
    ex_, ey_ = pp_ex * nx, pp_ey * ny
    x = np.arange(nx)[None, :]
    y = np.arange(ny)[:, None]
    xe = -ex_ / 2.0 + pp_ex * x
    ye = (ey_ / 2.0 - pp_ey) - pp_ey * y
    hc = hh * np.exp(1j * np.pi / lam / field_lens * (xe * xe + ye * ye))
    sx = int(math.floor(abs(cx / pp_ex) + 0.5)) * (1 if cx >= 0 else -1)     # C round: halves away from zero
    sy = int(math.floor(abs(cy / pp_ey) + 0.5)) * (1 if cy >= 0 else -1)
    he = _circshift(hc, -sx, sy)
    f_eye = eye_length * (field_lens - focus) / (eye_length + (field_lens - focus))
    eff = f_eye * eye_length / (f_eye - eye_length)
    r = np.sqrt(xe * xe + ye * ye)
    k2 = np.exp(1j * np.pi / lam / eff * (xe * xe + ye * ye))
    mask = (r < abs(lam * eff / (2.0 * max(pp_ex, pp_ey)))) & (r < pupil / 2.0)
    he = he * k2 * mask
    return np.abs(_fftw_shift(he))
