"""The reference-signature launchers (include/oh_reference_shims.h), driven
step for step the way HologramGenerator::Calc_Holo_GPU and encoding_GPU drive
them (HologramGenerator_GPU.cpp:211-231, 246-302, 338-368), against the oracle."""
import ctypes as C
import math

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, scenes
from oracle import depthmap as odm

pytestmark = pytest.mark.gpu


def _shims():
    L = _lib.lib()
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    L.cudaFFT.argtypes = [vp, i, i, vp, vp, i, C.c_bool]
    L.cudaDepthHoloKernel.argtypes = [vp, i, i, vp, vp, vp, vp, i, d, d, d, d, i, C.c_uint]
    L.cudaPropagation_AngularSpKernel.argtypes = [vp, i, i, vp, vp, d, d, d, d, d, d, d]
    L.cudaCropFringe.argtypes = [vp, i, i, vp, vp, i, i, i, i]
    L.cudaGetFringe.argtypes = [vp, i, i, vp, vp, i, i, d, d, d, d, d]
    L.cudaChangeDepthQuanKernel.argtypes = [vp, i, i, vp, vp, i, d, d, d, d, d]
    for f in ("cudaFFT", "cudaDepthHoloKernel", "cudaPropagation_AngularSpKernel", "cudaCropFringe", "cudaGetFringe",
              "cudaChangeDepthQuanKernel"):
        getattr(L, f).restype = None
    L.oh_shim_last_status.restype = C.c_int
    return L


def P(t):
    return C.c_void_p(t.data_ptr())


def test_cudafft_semantics(lib_built):
    L = _shims()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    x = np.random.default_rng(0).standard_normal((30, 40)) + 1j * np.random.default_rng(1).standard_normal((30, 40))
    tin = torch.from_numpy(x).cuda()
    tout = torch.zeros_like(tin)
    L.cudaFFT(st, 40, 30, P(tin), P(tout), -1, False)
    torch.cuda.synchronize()
    assert L.oh_shim_last_status() == 0
    ref = np.fft.fftshift(np.fft.fft2(np.fft.fftshift(x)))
    assert np.allclose(tout.cpu().numpy(), ref, atol=1e-10)
    # the input buffer holds the unshifted transform, as cuFFT leaves it there
    assert np.allclose(tin.cpu().numpy(), np.fft.fft2(np.fft.fftshift(x)), atol=1e-10)
    tin2 = torch.from_numpy(x).cuda()
    L.cudaFFT(st, 40, 30, P(tin2), P(tout), 1, True)
    torch.cuda.synchronize()
    assert np.allclose(tout.cpu().numpy(), np.fft.fftshift(np.fft.ifft2(np.fft.fftshift(x))), atol=1e-12)


def test_reference_gpu_driver_sequence(lib_built):
    """Calc_Holo_GPU + encoding_GPU through the six shims == oracle (pad 1)."""
    L = _shims()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ny, nx, nd = 54, 96, 10
    img, depth = scenes.depthmap_scene(77, ny, nx)
    near, far, lam, ppx, ppy, f = 0.2, 0.7, 532e-9, 8e-6, 8e-6, 1.0
    op = odm.DMParams(pnx=nx, pny=ny, ppx=ppx, ppy=ppy, lam=lam, near=near, far=far, num_of_depth=nd, pad=1,
                      transform_viewing_window=1, field_lens=f, rand_phase=complex(math.cos(1.1), math.sin(1.1)))
    dstep, lv = odm.depth_levels(op)
    zt = odm.transformed_levels(op)
    k = 2 * math.pi / lam
    ssx, ssy = nx * ppx, ny * ppy
    N = nx * ny
    d_img = torch.from_numpy(img).cuda()
    d_dimg = torch.from_numpy(depth).cuda()
    d_idx = torch.zeros(N, dtype=torch.float64, device="cuda")
    for dtr in range(nd):                              # change_depth_quan_GPU
        L.cudaChangeDepthQuanKernel(st, nx, ny, P(d_idx), P(d_dimg), dtr, lv[dtr] - dstep / 2.0, lv[dtr] + dstep / 2.0,
                                    float(nd), far, near)
    u_o = torch.zeros(N, dtype=torch.complex128, device="cuda")
    u_c = torch.zeros(N, dtype=torch.complex128, device="cuda")
    k_t = torch.zeros(N, dtype=torch.complex128, device="cuda")
    for dtr in range(1, nd + 1):
        z = zt[dtr - 1]
        u_o.zero_()
        L.cudaDepthHoloKernel(st, nx, ny, P(u_o), P(d_img), P(d_dimg), P(d_idx), dtr, op.rand_phase.real,
                              op.rand_phase.imag, math.cos(k * z), math.sin(k * z), 1, 256)
        k_t.zero_()
        L.cudaFFT(st, nx, ny, P(u_o), P(k_t), -1, False)
        L.cudaPropagation_AngularSpKernel(st, nx, ny, P(k_t), P(u_c), ppx, ppy, ssx, ssy, lam, k, -z)
    cx1, cx2, cy1, cy2 = odm.crop_window(nx, ny, (0, 1))
    k_t.zero_()
    L.cudaCropFringe(st, nx, ny, P(u_c), P(k_t), cx1, cx2, cy1, cy2)
    u_c.zero_()
    L.cudaFFT(st, nx, ny, P(k_t), P(u_c), 1, True)
    k_t.zero_()
    L.cudaGetFringe(st, nx, ny, P(u_c), P(k_t), 0, 1, ssx, ssy, ppx, ppy, math.pi)
    torch.cuda.synchronize()
    assert L.oh_shim_last_status() == 0
    got = k_t.cpu().numpy().real.reshape(ny, nx)
    ref = odm.generate(img, depth, op)[0]
    assert np.linalg.norm(got - ref) <= 1e-9 * np.linalg.norm(ref)
