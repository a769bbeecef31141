"""The learned surrogate through the C ABI: a U-Net (oh_unet_*) that maps an
RGB-D frame to the complex mid-plane field of the plain layered
angular-spectrum method, trained on the GPU by the library's own forward and
backward kernels.  No reference counterpart; the plain method it stands in
for is HologramGenerator::Calc_Holo_GPU (HologramGenerator_GPU.cpp:246-302).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import UnetConfig


def layer_shapes(in_ch=4, chans=(32, 64, 128, 256), out_ch=2):
    """(name, cin, cout, taps) of every layer in the flat parameter order."""
    L = []
    c_prev = in_ch
    for l, c in enumerate(chans):
        L += [(f"enc{l}a", c_prev, c, 9), (f"enc{l}b", c, c, 9)]
        c_prev = c
    for l in range(len(chans) - 2, -1, -1):
        L += [(f"dec{l}a", chans[l] + chans[l + 1], chans[l], 9), (f"dec{l}b", chans[l], chans[l], 9)]
    L.append(("head", chans[0], out_ch, 1))
    return L


def unflatten(flat: np.ndarray) -> dict:
    """Flat parameter array -> {name: (W [cout, taps, cin], b [cout])}."""
    out, o = {}, 0
    for name, cin, cout, taps in layer_shapes():
        nw = cout * taps * cin
        out[name] = (flat[o:o + nw].reshape(cout, taps, cin), flat[o + nw:o + nw + cout])
        o += nw + cout
    assert o == flat.size
    return out


def _stream(stream):
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return C.c_void_p(stream if isinstance(stream, int) else stream.cuda_stream)


class UNet:
    """Owns one oh_unet on a context's device."""

    def __init__(self, ctx: _lib.Context, max_batch=1, max_height=1024, max_width=1024, seed=1, out_scale=1.0,
                 depth_lut=None):
        cfg = UnetConfig()
        _lib.lib().oh_unet_config_default(C.byref(cfg))
        cfg.max_batch, cfg.max_height, cfg.max_width, cfg.seed, cfg.out_scale = (max_batch, max_height, max_width,
                                                                                 seed, out_scale)
        if depth_lut is not None:
            for i, v in enumerate(np.asarray(depth_lut, dtype=np.float32)):
                cfg.depth_lut[i] = float(v)
        h = C.c_void_p()
        _lib.call("oh_unet_create", ctx.handle, C.byref(cfg), C.byref(h))
        self.handle = h
        self.ctx = ctx
        self.n_params = int(_lib.lib().oh_unet_param_count(h))

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            _lib.lib().oh_unet_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        a = np.empty(self.n_params, dtype=np.float32)
        _lib.call("oh_unet_get_params", self.handle, a.ctypes.data_as(C.c_void_p))
        return a

    def set_params(self, flat: np.ndarray) -> None:
        a = np.ascontiguousarray(flat, dtype=np.float32)
        assert a.size == self.n_params
        _lib.call("oh_unet_set_params", self.handle, a.ctypes.data_as(C.c_void_p))

    def get_grads(self) -> np.ndarray:
        a = np.empty(self.n_params, dtype=np.float32)
        _lib.call("oh_unet_get_grads", self.handle, a.ctypes.data_as(C.c_void_p))
        return a

    def forward(self, rgbd, out=None, stream=None):
        """rgbd: uint8 device tensor [n, h, w, 4]; returns complex64 [n, h, w]."""
        import torch
        n, h, w, _ = rgbd.shape
        if out is None:
            out = torch.empty((n, h, w), dtype=torch.complex64, device=rgbd.device)
        _lib.call("oh_unet_forward", self.handle, C.c_void_p(rgbd.data_ptr()), n, h, w, C.c_void_p(out.data_ptr()),
                  _stream(stream))
        return out

    def compute_grads(self, rgbd, target, loss=None, stream=None):
        n, h, w, _ = rgbd.shape
        _lib.call("oh_unet_compute_grads", self.handle, C.c_void_p(rgbd.data_ptr()), C.c_void_p(target.data_ptr()),
                  n, h, w, C.c_void_p(loss.data_ptr()) if loss is not None else None, _stream(stream))

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
        _lib.call("oh_unet_adam_step", self.handle, lr, beta1, beta2, eps, _stream(stream))

    def train_step(self, rgbd, target, lr, loss=None, stream=None):
        n, h, w, _ = rgbd.shape
        _lib.call("oh_unet_train_step", self.handle, C.c_void_p(rgbd.data_ptr()), C.c_void_p(target.data_ptr()),
                  n, h, w, lr, C.c_void_p(loss.data_ptr()) if loss is not None else None, _stream(stream))


def scenes_rgbd(ctx: _lib.Context, seed: int, n: int, h: int, w: int, out=None, stream=None):
    """n seeded RGB-D frames on the device (oh_scene_rgbd): uint8 [n, h, w, 4]."""
    import torch
    if out is None:
        out = torch.empty((n, h, w, 4), dtype=torch.uint8, device="cuda")
    _lib.call("oh_scene_rgbd", ctx.handle, seed, n, h, w, C.c_void_p(out.data_ptr()), _stream(stream))
    return out


def mid_field(ctx: _lib.Context, p, z_mid: float, rgbd, out=None, stream=None):
    """The plain method's mid-plane field of one RGB-D frame (the training
    target): complex64 [pny, pnx]."""
    import torch
    if out is None:
        out = torch.empty((p.pny, p.pnx), dtype=torch.complex64, device=rgbd.device)
    _lib.call("oh_surrogate_mid_field", ctx.handle, C.byref(p), z_mid, C.c_void_p(rgbd.data_ptr()),
              C.c_void_p(out.data_ptr()), _stream(stream))
    return out


def generate(ctx: _lib.Context, net: UNet, p, z_mid: float, rgbd, check=False, psnr_threshold_db=40.0,
             fringe=None, field_mid=None, stream=None):
    """One frame through the surrogate (oh_surrogate_generate).  Returns
    (fringe, report dict)."""
    import torch
    sp = _lib.SurrogateParams()
    sp.dm = p
    sp.z_mid, sp.psnr_threshold_db, sp.check = z_mid, psnr_threshold_db, 1 if check else 0
    if fringe is None:
        fringe = torch.empty((p.pny, p.pnx), dtype=torch.float32, device=rgbd.device)
    rep = _lib.SurrogateReport()
    _lib.call("oh_surrogate_generate", ctx.handle, net.handle, C.byref(sp), C.c_void_p(rgbd.data_ptr()),
              C.c_void_p(fringe.data_ptr()), C.c_void_p(field_mid.data_ptr()) if field_mid is not None else None,
              C.byref(rep), _stream(stream))
    return fringe, {"checked": rep.checked, "fell_back": rep.fell_back, "psnr_db": rep.psnr_db,
                    "rel_err": rep.rel_err, "max_abs_err": rep.max_abs_err, "rms_err": rep.rms_err}


def train(ctx: _lib.Context, net: UNet, p, z_mid: float, samples: int, batch: int, lr: float, seed: int,
          log_every: int = 0, stream=None):
    """Train on `samples` seeded RGB-D frames of the plain method's geometry
    p (pny x pnx), `batch` frames per Adam step, targets from the plain
    mid-plane field, all on the GPU.  Frame i uses scene seed seed + i.
    Returns the per-step losses (device-side values copied at the end)."""
    import torch
    h, w = p.pny, p.pnx
    rgbd = torch.empty((batch, h, w, 4), dtype=torch.uint8, device="cuda")
    target = torch.empty((batch, h, w), dtype=torch.complex64, device="cuda")
    steps = samples // batch
    losses = torch.zeros(steps, dtype=torch.float32, device="cuda")
    for s in range(steps):
        scenes_rgbd(ctx, seed + s * batch, batch, h, w, out=rgbd, stream=stream)
        for b in range(batch):
            mid_field(ctx, p, z_mid, rgbd[b], out=target[b], stream=stream)
        net.train_step(rgbd, torch.view_as_real(target), lr, loss=losses[s:s + 1], stream=stream)
        if log_every and (s % log_every == 0):
            print(f"step {s}: loss {float(losses[s]):.4e}", flush=True)
    return losses.cpu().numpy()
