"""CPU oracle for LF-CGH — TEST INFRASTRUCTURE ONLY.

Restates fn_convertLightField2ComplexField.m:1-11 (OpenHolo_LFCGH) with
fn_myfft2.m (fftshift(fft2(ifftshift(.)))) in numpy: block (t, s) of the
(nt nv) x (ns nu) field is the centred FFT of view (t, s) times
exp(i phase).  MATLAB draws phase = 2 pi rand; here it is an input.  Parity
unpinned (no MATLAB here).
"""
from __future__ import annotations

import numpy as np


def lightfield_to_field(lf, phase):
    """lf, phase: (nt, ns, nv, nu) arrays."""
    lf = np.asarray(lf, dtype=np.float64)
    nt, ns, nv, nu = lf.shape
    out = np.zeros((nt * nv, ns * nu), np.complex128)
    for s in range(ns):
        for t in range(nt):
            view = lf[t, s] * np.exp(1j * np.asarray(phase[t, s], dtype=np.float64))
            out[t * nv:(t + 1) * nv, s * nu:(s + 1) * nu] = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(view)))
    return out
