"""CPU oracle for the encoders — TEST INFRASTRUCTURE ONLY.

numpy restatements of OpenHolo_Encoding/fn_encoding.m:29-98 (MATLAB,
1-based indices translated), fn_myfft2.m / fn_myifft2.m
(fftshift(fft2(ifftshift(.)))), the phase-only uint8 image of
OpenHolo_WRP/WRP_matlab_ver 1.0/Hologram_WRP.m:57-60 and ophNormalize
(OpenHolo_KETI/.../oph_common/oph_common.cpp:92-115).
"""
from __future__ import annotations

import numpy as np


def myfft2(a):
    return np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(a)))


def myifft2(a):
    return np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(a)))


def ssb(U, passband):
    ny, nx = U.shape
    AS = myfft2(U)
    if passband == "left":
        AS[:, nx // 2 - 1:] = 0
    elif passband == "right":
        AS[:, :nx // 2] = 0
    elif passband == "top":
        AS[ny // 2 - 1:, :] = 0
    elif passband == "bottom":
        AS[:ny // 2, :] = 0
    re = np.real(myifft2(AS))
    pos = re - re.min()
    return pos / pos.max()


def ni(U):
    ref = np.abs(U).max()
    inter = np.abs(U + ref) ** 2
    return inter / inter.max()


def p2a(U):
    return np.angle(U) + np.pi / (2 * np.pi)     # fn_encoding.m:57, operator precedence as written


def burckhardt(U):
    ny, nx = U.shape
    A1 = np.zeros((ny, nx)); A2 = np.zeros((ny, nx)); A3 = np.zeros((ny, nx))
    U = U / np.abs(U).max()
    phase = np.angle(U) + np.pi
    amp = np.abs(U)
    s3 = np.sqrt(3)
    i = (phase >= 0) & (phase < 2 * np.pi / 3)
    A1[i] = amp[i] * (np.cos(phase[i]) + np.sin(phase[i]) / s3)
    A2[i] = 2 * np.sin(phase[i]) / s3
    i = (phase >= 2 * np.pi / 3) & (phase < 4 * np.pi / 3)
    A2[i] = amp[i] * (np.cos(phase[i] - 2 * np.pi / 3) + np.sin(phase[i] - 2 * np.pi / 3) / s3)
    A3[i] = 2 * np.sin(phase[i] - 2 * np.pi / 3) / s3
    i = (phase >= 4 * np.pi / 3) & (phase < 2 * np.pi)
    A3[i] = amp[i] * (np.cos(phase[i] - 4 * np.pi / 3) + np.sin(phase[i] - 4 * np.pi / 3) / s3)
    A1[i] = 2 * np.sin(phase[i] - 4 * np.pi / 3) / s3
    out = np.zeros((ny, 3 * nx))
    out[:, 0::3] = A1; out[:, 1::3] = A2; out[:, 2::3] = A3
    return out


def two_phase(U):
    ny, nx = U.shape
    U = U / np.abs(U).max()
    amp = np.abs(U)
    phase = np.angle(U) + np.pi
    d = np.arccos(np.minimum(amp, 1.0))     # real part of MATLAB's acos for a rounding-level 1+eps
    out = np.zeros((ny, 2 * nx))
    out[:, 0::2] = phase + d
    out[:, 1::2] = phase - d
    return out


def phase_only_u8(U):
    ph = np.angle(U) + np.pi
    v = 255 * ph / ph.max()
    return np.clip(np.floor(v + 0.5), 0, 255).astype(np.uint8)   # MATLAB uint8(): round half away, saturate


def encode(U, kind):
    return {"real": lambda u: np.real(u), "p2a": p2a, "ni": ni, "burckhardt": burckhardt, "two_phase": two_phase,
            "ssb_left": lambda u: ssb(u, "left"), "ssb_right": lambda u: ssb(u, "right"),
            "ssb_top": lambda u: ssb(u, "top"), "ssb_bottom": lambda u: ssb(u, "bottom"),
            "phase_only_u8": phase_only_u8, "amplitude": np.abs}[kind](U)


def keti_normalize(src: np.ndarray) -> np.ndarray:
    """ophNormalize: float min/max, +0.5 rounding, vertical flip."""
    src = src.astype(np.float32)
    mn, mx = src.min(), src.max()
    v = ((src - mn) / (mx - mn)) * np.float32(255) + np.float32(0.5)
    return v.astype(np.uint32).astype(np.uint8)[::-1].copy()
