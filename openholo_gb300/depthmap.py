"""Depth-map CGH through the C ABI (oh_depthmap_generate), with a
HologramGenerator-shaped front end.

The class mirrors the operator interface of the reference's
HologramGenerator (OpenHolo_DepthMap/Hologram/HologramGenerator.h:130-149):
setMode / readConfig / initialize / GenerateHologram.  Frames are passed as
uint8 arrays instead of being loaded through Qt.  Only the GPU path exists:
setMode(True) (the reference's CPU mode) raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import DepthmapParams, OH_FP32, OH_FP64, OH_PHASE_ARRAY, OH_PHASE_REFERENCE, OH_PHASE_SEEDED


def _stream_ptr(stream):
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


def make_params(pnx=1920, pny=1080, ppx=8e-6, ppy=8e-6, lam=532e-9, near=0.30, far=0.35, num_of_depth=32,
                flag_change_depth_quantization=1, default_depth_quantization=256, transform_viewing_window=0,
                field_lens=1.0, pad=2, sig_location=(0, 1), phase_mode=OH_PHASE_REFERENCE, seed=0,
                rand_phase=1 + 0j, render_depth=None) -> DepthmapParams:
    p = DepthmapParams()
    _lib.lib().oh_depthmap_params_default(C.byref(p))
    p.pnx, p.pny, p.ppx, p.ppy, p.lambda_ = pnx, pny, ppx, ppy, lam
    p.near_depthmap, p.far_depthmap, p.num_of_depth = near, far, num_of_depth
    p.flag_change_depth_quantization = flag_change_depth_quantization
    p.default_depth_quantization = default_depth_quantization
    p.transform_viewing_window, p.field_lens, p.pad = transform_viewing_window, field_lens, pad
    p.sig_location_x, p.sig_location_y = sig_location
    p.phase_mode, p.seed = phase_mode, seed
    p.rand_phase_re, p.rand_phase_im = complex(rand_phase).real, complex(rand_phase).imag
    if render_depth is not None:
        arr = (C.c_int * len(render_depth))(*render_depth)
        p._render_keep = arr          # keep the array alive with the struct
        p.render_depth = C.cast(arr, C.POINTER(C.c_int))
        p.n_render_depth = len(render_depth)
    return p


def levels(p: DepthmapParams):
    """(lut[256] int16, z'[num_of_depth]) exactly as the library bins them."""
    lut = np.zeros(256, dtype=np.int16)
    z = np.zeros(p.num_of_depth, dtype=np.float64)
    _lib.call("oh_depthmap_levels", C.byref(p), lut.ctypes.data_as(C.c_void_p), z.ctypes.data_as(C.c_void_p))
    return lut, z


def generate(ctx: _lib.Context, p: DepthmapParams, img, depth, phase=None, precision="fp32",
             fringe=None, field=None, spectrum=None, stream=None):
    """Run one frame on device tensors (torch, uint8 [pny][pnx]).  Returns the
    fringe tensor (float32/float64 [pny][pnx]); `field` / `spectrum` may be
    given as preallocated complex tensors to receive the complex hologram and
    the accumulated spectrum."""
    import torch
    prec = OH_FP64 if precision == "fp64" else OH_FP32
    rdt = torch.float64 if prec == OH_FP64 else torch.float32
    if fringe is None:
        fringe = torch.empty((p.pny, p.pnx), dtype=rdt, device=img.device)
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
    _lib.call("oh_depthmap_generate", ctx.handle, prec, C.byref(p), ptr(img), ptr(depth), ptr(phase),
              ptr(fringe), ptr(field), ptr(spectrum), _stream_ptr(stream))
    return fringe


def propagate_field(ctx: _lib.Context, p: DepthmapParams, field, z: float, precision="fp32", fringe=None,
                    out_field=None, stream=None):
    """One complex source field (device tensor [pny][pnx]) as a single layer at
    distance z through the frame pipeline (oh_depthmap_propagate_field);
    returns the fringe."""
    import torch
    prec = OH_FP64 if precision == "fp64" else OH_FP32
    if fringe is None:
        fringe = torch.empty((p.pny, p.pnx), dtype=torch.float64 if prec == OH_FP64 else torch.float32,
                             device=field.device)
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
    _lib.call("oh_depthmap_propagate_field", ctx.handle, prec, C.byref(p), ptr(field), z, ptr(fringe), ptr(out_field),
              None, _stream_ptr(stream))
    return fringe


def generate_batch(ctx: _lib.Context, frames, precision="fp32", graph=False, stream=None):
    """Run a list of frames in one call (oh_depthmap_generate_batch).  Each
    entry is (params, img, depth, fringe[, phase[, field]]) with device
    tensors; fringe (and field, complex, when given) receive the result.  graph=True
    captures the batch into a CUDA graph on the first call and replays it on
    later calls with the same frames (same parameters and tensors)."""
    prec = OH_FP64 if precision == "fp64" else OH_FP32
    arr = _frame_array(frames)
    _lib.call("oh_depthmap_generate_batch", ctx.handle, prec, arr, len(frames),
              _lib.BATCH_GRAPH if graph else 0, _stream_ptr(stream))


def _frame_array(frames):
    """Entries (params, img, depth, fringe[, phase[, field]]) of device tensors."""
    arr = (_lib.DepthmapFrame * len(frames))()
    for i, fr in enumerate(frames):
        p, img, depth, fringe = fr[:4]
        phase = fr[4] if len(fr) > 4 else None
        field = fr[5] if len(fr) > 5 else None
        arr[i].params = p
        arr[i].img = img.data_ptr()
        arr[i].depth = depth.data_ptr()
        arr[i].phase = phase.data_ptr() if phase is not None else None
        arr[i].fringe = fringe.data_ptr()
        arr[i].field = field.data_ptr() if field is not None else None
    return arr


def set_batch_mode(ctx: _lib.Context, persistent: bool):
    """True: batches the persistent kernel carries run as one launch of it
    (the default); False: every batch runs as per-frame launches."""
    _lib.call("oh_ctx_set_depthmap_batch_mode", ctx.handle, 1 if persistent else 0)


def autotune_batch(ctx: _lib.Context, frames, reps=2, stream=None):
    """Tune the persistent batch kernel on the square frames of `frames`
    (oh_depthmap_autotune_batch); later batches on ctx use the result."""
    arr = _frame_array(frames)
    _lib.call("oh_depthmap_autotune_batch", ctx.handle, arr, len(frames), reps, _stream_ptr(stream))


BATCH_SETTINGS = ("ctas_per_sm", "lag", "col_w", "row_pairs", "col_blocks", "out_rows")


def batch_tuning(ctx: _lib.Context, padded_len: int) -> dict:
    """Settings batches of this padded length use (oh_depthmap_batch_tuning)."""
    v = (C.c_int * 6)()
    ms = C.c_double()
    _lib.call("oh_depthmap_batch_tuning", ctx.handle, padded_len, v, C.byref(ms))
    return {**dict(zip(BATCH_SETTINGS, list(v))), "ms": ms.value}


def set_autotune_file(ctx: _lib.Context, path):
    _lib.call("oh_ctx_set_autotune_file", ctx.handle, None if path is None else str(path).encode())


def generate_host(ctx: _lib.Context, p: DepthmapParams, img: np.ndarray, depth: np.ndarray,
                  phase: np.ndarray | None = None, precision="fp32", out: np.ndarray | None = None, stream=None):
    """Host buffers in and out (oh_depthmap_generate_host)."""
    prec = OH_FP64 if precision == "fp64" else OH_FP32
    if out is None:
        out = np.empty((p.pny, p.pnx), dtype=np.float64 if prec == OH_FP64 else np.float32)
    img = np.ascontiguousarray(img, dtype=np.uint8)
    depth = np.ascontiguousarray(depth, dtype=np.uint8)
    ph = None if phase is None else np.ascontiguousarray(phase, dtype=np.float32)
    vp = lambda a: a.ctypes.data_as(C.c_void_p) if a is not None else None
    _lib.call("oh_depthmap_generate_host", ctx.handle, prec, C.byref(p), vp(img), vp(depth), vp(ph), vp(out),
              _stream_ptr(stream))
    return out


def read_config(path: str) -> DepthmapParams:
    p = DepthmapParams()
    _lib.call("oh_depthmap_read_config", str(path).encode(), C.byref(p))
    # copy the render list out of thread-local library storage
    lst = [p.render_depth[i] for i in range(p.n_render_depth)]
    arr = (C.c_int * len(lst))(*lst)
    p._render_keep = arr
    p.render_depth = C.cast(arr, C.POINTER(C.c_int))
    return p


@dataclass
class _Frame:
    img: np.ndarray
    depth: np.ndarray


class HologramGenerator:
    """Qt-free mirror of HologramGenerator (HologramGenerator.h:130-149)."""

    def __init__(self, device: int = 0):
        self.isCPU_ = False
        self.params_ = None
        self.ctx = _lib.Context(device)
        self.u255_fringe_ = None
        self.precision = "fp64"     # the reference computes in double

    def setMode(self, isCPU: bool) -> None:
        if isCPU:
            raise NotImplementedError("this library has no CPU path; the hologram is computed on the GPU")
        self.isCPU_ = False

    def readConfig(self, path: str = "config_openholo.txt") -> bool:
        try:
            self.params_ = read_config(path)
        except _lib.OhError:
            return False
        return True

    def initialize(self) -> None:
        if self.params_ is None:
            raise RuntimeError("readConfig() first")

    def GenerateHologram(self, img: np.ndarray, depth: np.ndarray) -> np.ndarray:
        """One static frame: Calc_Holo_by_Depth + Encoding_Symmetrization;
        returns u255_fringe_ (real fringe before uint8 normalisation)."""
        self.u255_fringe_ = generate_host(self.ctx, self.params_, img, depth, precision=self.precision)
        return self.u255_fringe_


def reconstruct_eye(ctx: _lib.Context, fringe, pnx: int, pny: int, ppx: float, ppy: float, lam: float,
                    field_lens: float, eye_length: float, pupil_diameter: float, eye_center=(0.0, 0.0),
                    focus_distance: float = 0.5, pixel_scale: int = 1, precision="fp64", stream=None):
    """Eye-model reconstruction of a fringe (HologramGenerator::ReconstructImage,
    one frame; oh_reconstruct_eye).  fringe: device tensor [pny][pnx] (real).
    Returns the retina-plane magnitude [pny/s][pnx/s].  A focus sweep is one
    call per focus distance."""
    import torch
    prec = OH_FP64 if precision == "fp64" else OH_FP32
    dt = torch.float64 if prec == OH_FP64 else torch.float32
    f = fringe.to(dt).contiguous()
    out = torch.empty((pny // pixel_scale, pnx // pixel_scale), dtype=dt, device=f.device)
    p = _lib.EyeParams(pnx, pny, ppx, ppy, lam, field_lens, pixel_scale, eye_length, pupil_diameter,
                       eye_center[0], eye_center[1], focus_distance)
    _lib.call("oh_reconstruct_eye", ctx.handle, prec, C.byref(p), C.c_void_p(f.data_ptr()),
              C.c_void_p(out.data_ptr()), _stream_ptr(stream))
    return out
