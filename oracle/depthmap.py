"""CPU oracle for the layered angular-spectrum depth-map CGH — TEST
INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline may import this module; the product never does.

A float64 numpy restatement of the reference's depth-map path
(OpenHolo_DepthMap/Hologram/src):

  GetDepthValues              HologramGenerator.cpp:391-417
  change_depth_quan_CPU       HologramGenerator_CPU.cpp:74-103
  prepare_inputdata_CPU       HologramGenerator_CPU.cpp:44-67
  TransformViewingWindow      HologramGenerator.cpp:423-435
  Calc_Holo_CPU               HologramGenerator_CPU.cpp:117-177
  Propagation_AngularSpectrum HologramGenerator_CPU.cpp:186-218, HologramKernel.cu:75-103
  Encoding_Symmetrization     HologramGenerator.cpp:481-522
  encoding_CPU / getFringe    HologramGenerator_CPU.cpp:231-270, HologramKernel.cu:121-166
  get_shift_phase_value       HologramGenerator_CPU.cpp:367-408
  fftShift (GPU convention)   HologramKernel.cu:10-34  == numpy.fft.fftshift
  Write_Result_image          HologramGenerator.cpp:528-565

Layers are accumulated sequentially (the reference's OpenMP layer loop races
on U_complex_, HologramGenerator_CPU.cpp:129/215).  FFTW is replaced by
numpy/scipy pocketfft (FFTW and Qt are not available).  At pad 1 the oracle
reproduces the reference's own GPU kernels (HologramKernel.cu, compiled from
its source and run in the order of Calc_Holo_GPU / encoding_GPU with cuFFT)
to FP64 rounding: tests/test_dm_reference_golden.py against the fixtures in
tests/golden/dm_reference_gpu.npz.

Extensions beyond the reference, used by the 1920x1080 / 32-layer workload:
  pad = 2   the layer field is embedded, centred (offset n/2), in a 2x grid;
            the reference's frequency grid, transfer function and crop window
            are evaluated on that grid; after the inverse transform the
            centre pny x pnx region is kept and the shift phase of the
            original grid applied.
  phase     per-pixel source phase (array, or the seeded SplitMix64 stream).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

try:
    import scipy.fft as _sfft
except Exception:  # pragma: no cover
    _sfft = None


@dataclass
class DMParams:
    pnx: int = 1920
    pny: int = 1080
    ppx: float = 8e-6
    ppy: float = 8e-6
    lam: float = 532e-9
    field_lens: float = 1000e-3
    near: float = 0.30
    far: float = 0.35
    num_of_depth: int = 32
    flag_change_depth_quantization: int = 1
    default_depth_quantization: int = 256
    transform_viewing_window: int = 0
    pad: int = 2
    sig_location: tuple = (0, 1)
    rand_phase: complex = 1 + 0j
    render_depth: list | None = None     # 1-based levels; None = all
    extra: dict = field(default_factory=dict)


def depth_levels(p: DMParams):
    """GetDepthValues (HologramGenerator.cpp:391-408): levels by repeated
    addition while val <= far.  When rounding ends the list one short of
    num_of_depth the addition is continued (the reference would index past
    the end of dlevel_)."""
    near = min(p.near, p.far)
    far = max(p.near, p.far)
    nd = p.num_of_depth
    if nd > 1:
        dstep = (far - near) / (nd - 1)
        lv = []
        val = near
        while val <= far and len(lv) < nd:
            lv.append(val)
            val += dstep
        while len(lv) < nd:
            lv.append(val)
            val += dstep
    else:
        dstep = (far + near) / 2
        lv = [far - near]
    return dstep, lv


def depth_lut(p: DMParams) -> np.ndarray:
    """Layer number per depth byte (256 entries), by the binning of
    change_depth_quan_CPU (HologramGenerator_CPU.cpp:82-99) / the
    FLAG_CHANGE_DEPTH_QUANTIZATION==0 rule (prepare_inputdata_CPU :64-65)."""
    near = min(p.near, p.far)
    far = max(p.near, p.far)
    dstep, lv = depth_levels(p)
    nd = p.num_of_depth
    lut = np.zeros(256, dtype=np.int64)
    for b in range(256):
        if p.flag_change_depth_quantization == 1:
            dmap_src = float(b) / 255.0
            dmap = (1 - dmap_src) * (far - near) + near
            idx = 0
            for dtr in range(nd):
                t = lv[dtr]
                d1 = t - dstep / 2.0
                d2 = t + dstep / 2.0
                if dtr < nd - 1:
                    hit = (1 if dmap >= d1 else 0) * (1 if dmap < d2 else 0)
                else:
                    hit = (1 if dmap >= d1 else 0) * (1 if dmap <= d2 else 0)
                idx += hit * (dtr + 1)
        else:
            idx = p.default_depth_quantization - b
        lut[b] = idx
    return lut


def transformed_levels(p: DMParams) -> list:
    """TransformViewingWindow (HologramGenerator.cpp:423-435) when enabled,
    else the levels themselves."""
    _, lv = depth_levels(p)
    if p.transform_viewing_window:
        f = p.field_lens
        return [-f * d / (d - f) for d in lv]
    return list(lv)


def crop_window(nx: int, ny: int, sig_location):
    """Encoding_Symmetrization (HologramGenerator.cpp:486-514), 0-based."""
    if sig_location[1] == 0:
        cropy1, cropy2 = 1, ny
    else:
        cropy = ny // 2
        cropy1 = cropy - cropy // 2
        cropy2 = cropy1 + cropy - 1
    if sig_location[0] == 0:
        cropx1, cropx2 = 1, nx
    else:
        cropx = nx // 2
        cropx1 = cropx - cropx // 2
        cropx2 = cropx1 + cropx - 1
    return cropx1 - 1, cropx2 - 1, cropy1 - 1, cropy2 - 1


def _fft2(a, inverse=False, workers=None):
    if _sfft is not None:
        return _sfft.ifft2(a, workers=workers) if inverse else _sfft.fft2(a, workers=workers)
    return np.fft.ifft2(a) if inverse else np.fft.fft2(a)


def centred_fft2(a, inverse=False, workers=None):
    """fftShift . FFT . fftShift of HologramKernel.cu:189-227 (shift by
    floor(n/2) on both sides; the inverse is normalised by 1/N as
    bNormalized=true / fftwShift(.., true) do)."""
    return np.fft.fftshift(_fft2(np.fft.fftshift(a), inverse, workers))


def transfer_function(p: DMParams, Px: int, Py: int, d: float) -> np.ndarray:
    """H = exp(i k d sqrt(1 - (lambda fx)^2 - (lambda fy)^2)) on the
    reference's grid: fx = -1/(2ppx) + x/ssx, fy = 1/(2ppy) - 1/ssy - y/ssy
    (HologramGenerator_CPU.cpp:196-216).  The mask (fx^2+fy^2) < k^2 is
    always true there and is kept for fidelity."""
    k = 2 * math.pi / p.lam
    ssx, ssy = Px * p.ppx, Py * p.ppy
    x = np.arange(Px, dtype=np.float64)
    y = np.arange(Py, dtype=np.float64)
    fxx = (-1.0 / (2.0 * p.ppx)) + (1.0 / ssx) * x
    fyy = (1.0 / (2.0 * p.ppy)) - (1.0 / ssy) - (1.0 / ssy) * y
    sval = np.sqrt(1 - (p.lam * fxx[None, :]) ** 2 - (p.lam * fyy[:, None]) ** 2)
    sval = sval * (k * d)
    H = np.exp(1j * sval)
    mask = (fxx[None, :] ** 2 + fyy[:, None] ** 2) < (k * k)
    return np.where(mask, H, 0)


def source_field(img: np.ndarray, phase: np.ndarray | None) -> np.ndarray:
    """img/255 * alpha (prepare_inputdata_CPU :59-61) times exp(i phase)."""
    amp = img.astype(np.float64) / 255.0 * (img > 0)
    if phase is None:
        return amp.astype(np.complex128)
    return amp * np.exp(1j * phase.astype(np.float64))


def calc_holo(img, depth, p: DMParams, phase=None, workers=None, layers=None):
    """Accumulated spectrum U (Py x Px) of Calc_Holo_CPU on the (padded) grid.
    `layers` restricts the loop to a subset of render entries (CPU baseline
    sampling)."""
    pny, pnx = img.shape
    assert (pny, pnx) == (p.pny, p.pnx)
    P = p.pad
    Px, Py = P * pnx, P * pny
    ox, oy = (Px - pnx) // 2, (Py - pny) // 2
    k = 2 * math.pi / p.lam
    lut = depth_lut(p)
    idx = lut[depth]
    src = source_field(img, phase)
    zt = transformed_levels(p)
    render = p.render_depth if p.render_depth is not None else list(range(1, p.num_of_depth + 1))
    if layers is not None:
        render = [render[i] for i in layers]
    U = np.zeros((Py, Px), dtype=np.complex128)
    u = np.zeros((Py, Px), dtype=np.complex128)
    for dtr in render:
        m = idx == dtr
        if not np.any(m & (img > 0)):
            continue                      # empty layer (HologramGenerator_CPU.cpp:145)
        z = zt[dtr - 1]
        carrier = complex(math.cos(k * z), math.sin(k * z))
        u[...] = 0
        u[oy:oy + pny, ox:ox + pnx] = np.where(m, src, 0) * p.rand_phase * carrier
        S = centred_fft2(u, workers=workers)
        U += transfer_function(p, Px, Py, -z) * S
    return U


def encode_symmetrization(U, p: DMParams, workers=None, return_field=False):
    """encoding_CPU (HologramGenerator_CPU.cpp:231-270) on the (padded) grid,
    then the centre pny x pnx region: fringe = Re(h * shift_phase)."""
    Py, Px = U.shape
    pny, pnx = p.pny, p.pnx
    ox, oy = (Px - pnx) // 2, (Py - pny) // 2
    cx1, cx2, cy1, cy2 = crop_window(Px, Py, p.sig_location)
    Uc = np.zeros_like(U)
    Uc[cy1:cy2 + 1, cx1:cx2 + 1] = U[cy1:cy2 + 1, cx1:cx2 + 1]
    h = centred_fft2(Uc, inverse=True, workers=workers)[oy:oy + pny, ox:ox + pnx]
    shift = np.ones((pny, pnx), dtype=np.complex128)
    ssx, ssy = pnx * p.ppx, pny * p.ppy
    if p.sig_location[1] != 0:
        r = np.arange(pny, dtype=np.float64)
        yy = (ssy / 2.0) - p.ppy * r - p.ppy
        ph = 2 * math.pi * (yy / (4 * p.ppy)) if p.sig_location[1] == 1 else 2 * math.pi * (-yy / (4 * p.ppy))
        shift = shift * np.exp(1j * ph)[:, None]
    if p.sig_location[0] != 0:
        c = np.arange(pnx, dtype=np.float64)
        xx = (-ssx / 2.0) - p.ppx * c - p.ppx
        ph = 2 * math.pi * (-xx / (4 * p.ppx)) if p.sig_location[0] == -1 else 2 * math.pi * (xx / (4 * p.ppx))
        shift = shift * np.exp(1j * ph)[None, :]
    hs = h * shift
    if return_field:
        return hs.real.copy(), hs
    return hs.real.copy()


def generate(img, depth, p: DMParams, phase=None, workers=None):
    """Full frame: (fringe, complex field, spectrum U)."""
    U = calc_holo(img, depth, p, phase=phase, workers=workers)
    fringe, field = encode_symmetrization(U, p, workers=workers, return_field=True)
    return fringe, field, U


def normalize_u8(fringe: np.ndarray) -> np.ndarray:
    """Write_Result_image (HologramGenerator.cpp:543-559): min/max scan with
    the reference's if / else-if update, then truncating conversion."""
    flat = fringe.ravel()
    mn = mx = flat[0]
    # the else-if of the reference can only miss a new max on the element
    # that set a new min, which cannot also be a new max: plain min/max
    mn = flat.min()
    mx = flat.max()
    return ((flat - mn) / (mx - mn) * 255).astype(np.uint32).astype(np.uint8).reshape(fringe.shape)
