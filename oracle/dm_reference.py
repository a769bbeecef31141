"""The reference's own depth-map GPU kernels, run in the reference's call
sequence — TEST INFRASTRUCTURE ONLY.  tests/golden/make_golden_depthmap.py uses it to
write golden fixtures, and tests/test_reference_gpu_gpu.py to compare the
library with it at full size and to time it as a baseline; nothing in the
product or the benchmark executes it.

oracle/build.py compiles OpenHolo_DepthMap/Hologram/src/HologramKernel.cu
(from the reference tree, unchanged) into oracle/_ref/dm_ref.cubin for
sm_103a.  This module loads that cubin through the CUDA driver API into the
current (PyTorch) context and issues its six kernels exactly as the
reference's host code does, with the reference's launch shape (512-thread
blocks, one thread per pixel, HologramKernel.cu:8):

  change_depth_quan_GPU          HologramGenerator_GPU.cpp:211-233
  Calc_Holo_GPU                  HologramGenerator_GPU.cpp:246-300
  Propagation_AngularSpectrum_GPU HologramGenerator_GPU.cpp:311-325
  Encoding_Symmetrization        HologramGenerator.cpp:481-522
  encoding_GPU                   HologramGenerator_GPU.cpp:338-369
  cudaFFT                        HologramKernel.cu:189-227

cudaFFT's cufftExecZ2Z is issued through torch.fft (PyTorch's CUDA FFT is
cuFFT): fft2 for CUFFT_FORWARD and ifft2(norm="forward") for the unnormalised
CUFFT_INVERSE.  Host-side values (depth levels, viewing-window transform,
carrier phase, crop window) follow the reference's host code, which
oracle/depthmap.py restates (GetDepthValues, TransformViewingWindow,
Encoding_Symmetrization); the carrier phase exp(i k z) is evaluated with the
host libm as the reference's exponent_complex does.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

from . import depthmap as odm

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "dm_ref.cubin"
THREADS = 512                                   # kBlockThreads, HologramKernel.cu:8

# mangled entry names as ptxas reports them for HologramKernel.cu
ENTRIES = {
    "fftShift": "_Z8fftShiftiiiP7double2S0_b",
    "depth_sources": "_Z20depth_sources_kernelP7double2PhS1_Pdiddddiiij",
    "propagation": "_Z28propagation_angularsp_kernelP7double2S0_iiddddddd",
    "cropFringe": "_Z10cropFringeiiP7double2S0_iiii",
    "getFringe": "_Z9getFringeiiP7double2S0_iiddddd",
    "change_depth_quan": "_Z24change_depth_quan_kernelPdPhiiiddddd",
}


class _Driver:
    def __init__(self, cubin: Path, entries: dict | None = None):
        import torch
        if not cubin.exists():
            raise FileNotFoundError(f"{cubin} is missing: build it with oracle/build.py where the reference tree is")
        torch.zeros(1, device="cuda")                # make PyTorch's primary context current
        self.cu = C.CDLL("libcuda.so.1")
        self._ok(self.cu.cuInit(0), "cuInit")
        ctx = C.c_void_p()
        self._ok(self.cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self.mod = C.c_void_p()
        self._ok(self.cu.cuModuleLoad(C.byref(self.mod), str(cubin).encode()), "cuModuleLoad")
        self.fn = {}
        for k, name in (entries or ENTRIES).items():
            f = C.c_void_p()
            self._ok(self.cu.cuModuleGetFunction(C.byref(f), self.mod, name.encode()), "cuModuleGetFunction " + name)
            self.fn[k] = f
        self.cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                           C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p]

    @staticmethod
    def _ok(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def launch2d(self, name, grid, block, *args):
        """Launch `name` with a 2-D grid and block (the point-cloud kernel)."""
        import torch
        vals = [a if isinstance(a, C._SimpleCData) else C.c_void_p(a) for a in args]
        ptrs = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        self._ok(self.cu.cuLaunchKernel(self.fn[name], grid[0], grid[1], 1, block[0], block[1], 1, 0, stream, ptrs,
                                        None), "cuLaunchKernel " + name)

    def launch(self, name, n, *args):
        import torch
        vals = [a if isinstance(a, C._SimpleCData) else C.c_void_p(a) for a in args]
        ptrs = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
        grid = (n + THREADS - 1) // THREADS
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        self._ok(self.cu.cuLaunchKernel(self.fn[name], grid, 1, 1, THREADS, 1, 1, 0, stream, ptrs, None),
                 "cuLaunchKernel " + name)


class ReferenceGPU:
    """One HologramGenerator in GPU mode: its device buffers (init_GPU,
    HologramGenerator_GPU.cpp:157-186) and the steps of one frame."""

    def __init__(self, p: odm.DMParams):
        import torch
        self.t = torch
        self.p = p
        self.d = _Driver(CUBIN)
        n = p.pnx * p.pny
        dev = "cuda"
        self.img = torch.zeros(n, dtype=torch.uint8, device=dev)
        self.dimg = torch.zeros(n, dtype=torch.uint8, device=dev)
        self.depth_index = torch.zeros(n, dtype=torch.float64, device=dev)
        self.u_o = torch.zeros(n, dtype=torch.complex128, device=dev)
        self.u_complex = torch.zeros(n, dtype=torch.complex128, device=dev)
        self.k_temp = torch.zeros(n, dtype=torch.complex128, device=dev)
        self.k = 2 * math.pi / p.lam                 # HologramGenerator.cpp:107
        self.ss = (p.pnx * p.ppx, p.pny * p.ppy)     # HologramGenerator.cpp:148-149

    def _fft(self, src, dst, direction, normalized=False):
        """cudaFFT(in=src, out=dst): shift src->dst, Z2Z dst->src, shift
        src->dst (normalised by nx*ny when asked)."""
        p, t = self.p, self.t
        n = p.pnx * p.pny
        self.d.launch("fftShift", n, C.c_int(n), C.c_int(p.pnx), C.c_int(p.pny), src.data_ptr(), dst.data_ptr(),
                      C.c_bool(False))
        g = dst.view(p.pny, p.pnx)
        r = t.fft.fft2(g) if direction == -1 else t.fft.ifft2(g, norm="forward")
        src.view(p.pny, p.pnx).copy_(r)
        self.d.launch("fftShift", n, C.c_int(n), C.c_int(p.pnx), C.c_int(p.pny), src.data_ptr(), dst.data_ptr(),
                      C.c_bool(bool(normalized)))

    def generate(self, img: np.ndarray, depth: np.ndarray):
        """Returns (u255 fringe float64 [pny][pnx], accumulated spectrum
        complex128 [pny][pnx]) for one frame."""
        p, t = self.p, self.t
        assert img.shape == (p.pny, p.pnx) and depth.shape == img.shape
        n = p.pnx * p.pny
        self.img.copy_(t.from_numpy(np.ascontiguousarray(img).ravel()))      # prepare_inputdata_GPU
        self.dimg.copy_(t.from_numpy(np.ascontiguousarray(depth).ravel()))
        dstep, lv = odm.depth_levels(p)                                      # GetDepthValues
        nd = p.num_of_depth
        if p.flag_change_depth_quantization == 1:                            # change_depth_quan_GPU
            self.depth_index.zero_()
            for dtr in range(nd):
                d1 = lv[dtr] - dstep / 2.0
                d2 = lv[dtr] + dstep / 2.0
                self.d.launch("change_depth_quan", n, self.depth_index.data_ptr(), self.dimg.data_ptr(),
                              C.c_int(p.pnx), C.c_int(p.pny), C.c_int(dtr), C.c_double(d1), C.c_double(d2),
                              C.c_double(float(nd)), C.c_double(p.far), C.c_double(p.near))
        zt = odm.transformed_levels(p)                                       # TransformViewingWindow
        self.u_complex.zero_()                                               # Calc_Holo_GPU
        render = p.render_depth if p.render_depth is not None else list(range(1, nd + 1))
        ra, rb = complex(p.rand_phase).real, complex(p.rand_phase).imag
        for dtr in render:
            z = zt[dtr - 1]
            ca, cb = math.exp(0.0) * math.cos(self.k * z), math.exp(0.0) * math.sin(self.k * z)
            self.u_o.zero_()
            self.d.launch("depth_sources", n, self.u_o.data_ptr(), self.img.data_ptr(), self.dimg.data_ptr(),
                          self.depth_index.data_ptr(), C.c_int(dtr), C.c_double(ra), C.c_double(rb),
                          C.c_double(ca), C.c_double(cb), C.c_int(p.pnx), C.c_int(p.pny),
                          C.c_int(p.flag_change_depth_quantization), C.c_uint(p.default_depth_quantization))
            self.k_temp.zero_()
            self._fft(self.u_o, self.k_temp, -1)
            self.d.launch("propagation", n, self.k_temp.data_ptr(), self.u_complex.data_ptr(), C.c_int(p.pnx),
                          C.c_int(p.pny), C.c_double(p.ppx), C.c_double(p.ppy), C.c_double(self.ss[0]),
                          C.c_double(self.ss[1]), C.c_double(p.lam), C.c_double(self.k), C.c_double(-z))
        spectrum = self.u_complex.view(p.pny, p.pnx).cpu().numpy().copy()
        cx1, cx2, cy1, cy2 = odm.crop_window(p.pnx, p.pny, p.sig_location)  # Encoding_Symmetrization
        self.k_temp.zero_()                                                  # encoding_GPU
        self.d.launch("cropFringe", n, C.c_int(p.pnx), C.c_int(p.pny), self.u_complex.data_ptr(),
                      self.k_temp.data_ptr(), C.c_int(cx1), C.c_int(cx2), C.c_int(cy1), C.c_int(cy2))
        self.u_complex.zero_()
        self._fft(self.k_temp, self.u_complex, 1, normalized=True)
        self.k_temp.zero_()
        self.d.launch("getFringe", n, C.c_int(p.pnx), C.c_int(p.pny), self.u_complex.data_ptr(),
                      self.k_temp.data_ptr(), C.c_int(p.sig_location[0]), C.c_int(p.sig_location[1]),
                      C.c_double(self.ss[0]), C.c_double(self.ss[1]), C.c_double(p.ppx), C.c_double(p.ppy),
                      C.c_double(math.pi))
        fringe = self.k_temp.view(p.pny, p.pnx).real.cpu().numpy().copy()
        t.cuda.synchronize()
        return fringe, spectrum
