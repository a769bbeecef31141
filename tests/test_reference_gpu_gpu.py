"""The library against the reference's own GPU code at the benchmark sizes,
and the reference's GPU timings as baselines.

- Depth map: the reference's HologramKernel.cu kernels, compiled from its
  source (oracle/_ref/dm_ref.cubin) and issued in the order of Calc_Holo_GPU
  / encoding_GPU (oracle/dm_reference.py: FP64, cuFFT Z2Z, pad 1, one
  constant reference phase), on a 1920x1080 frame with 32 levels.  The
  library's FP64 mode must match it to 1e-7 relative, its FP32 mode to 1e-3.
- Point cloud: the reference's ophKernelCghPointCloud_cuda, compiled from
  ophgen_pointcloud_gpu.cpp (oracle/_ref/pc_ref.cubin) and launched as
  ophGenCghPointCloud_cuda does (oracle/pc_reference_gpu.py), on 1024x1024
  pixels and 5000 points.  It evaluates k r in float (k r ~ 1.2e6 rad, so
  each term carries up to about 0.06 rad of phase rounding, and the sum
  about that much relative error): its fringe is compared with the
  library's FP64 one at a bound that holds that noise (0.1 relative; measured
  0.057), and its own error is printed.

Each test prints one JSON line with the reference's and the library's
times (CUDA events, after a warm-up; the depth-map reference time is the
wall clock of its host-driven call sequence, which copies its inputs in and
its spectrum and fringe out).  Skipped when the reference objects were not
built (they are built by oracle/build.py where the reference tree is).
"""
import ctypes as C
import json
import time

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, depthmap as dm, scenes
from openholo_gb300._lib import PcParams
from oracle import depthmap as odm

pytestmark = pytest.mark.gpu


def S():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def errs(got, ref):
    d = np.asarray(got) - ref
    return float(np.linalg.norm(d) / np.linalg.norm(ref)), float(np.abs(d).max() / np.abs(ref).max())


def events_ms(fn, reps):
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def test_depthmap_1920x1080_L32_vs_reference_gpu(ctx, dev):
    from oracle import dm_reference as dref
    if not dref.CUBIN.exists():
        pytest.skip("reference depth-map kernels not built (oracle/build.py needs the reference tree)")
    ny, nx, L = 1080, 1920, 32
    img, depth = scenes.depthmap_scene(2024, ny, nx)
    op = odm.DMParams(pnx=nx, pny=ny, num_of_depth=L, pad=1, transform_viewing_window=1)
    ref = dref.ReferenceGPU(op)
    ref.generate(img, depth)                               # warm-up (cuFFT plans)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        ref_fringe, ref_spec = ref.generate(img, depth)
    ref_ms = (time.perf_counter() - t0) * 1e3 / reps
    p = dm.make_params(pnx=nx, pny=ny, num_of_depth=L, pad=1, transform_viewing_window=1,
                       field_lens=op.field_lens, phase_mode=dm.OH_PHASE_REFERENCE)
    ti, td = torch.from_numpy(img).to(dev), torch.from_numpy(depth).to(dev)
    out = {"workload": "depth map 1920x1080, 32 levels, pad 1, reference phase mode",
           "reference_gpu_fp64_ms_per_frame": ref_ms}
    for precision, tol in (("fp64", 1e-7), ("fp32", 1e-3)):
        fr = torch.empty((ny, nx), dtype=torch.float64 if precision == "fp64" else torch.float32, device=dev)
        run = lambda: dm.generate(ctx, p, ti, td, precision=precision, fringe=fr)
        ms = events_ms(run, 5)
        rel, mx = errs(fr.cpu().numpy().astype(np.float64), ref_fringe)
        out[f"library_{precision}_ms_per_frame"] = ms
        out[f"library_{precision}_vs_reference_gpu"] = {"rel": rel, "max_abs_rel": mx}
        assert rel < tol and mx < 10 * tol, (precision, rel, mx)
    print(json.dumps(out))


def test_pointcloud_1024x1024_5000pts_vs_reference_gpu(ctx, dev):
    from oracle import pc_reference_gpu as pref
    if not pref.CUBIN.exists():
        pytest.skip("reference point-cloud kernel not built (oracle/build.py needs the reference tree)")
    n, nx, ny = 5000, 1024, 1024
    pts = scenes.pointcloud_scene(11, n).astype(np.float32)
    spec = {"scale_x": 1.0, "scale_y": 1.0, "scale_z": 1.0, "offset_depth": 0.0, "pitch_x": 8e-6, "pitch_y": 8e-6,
            "nx": nx, "ny": ny, "lambda": 532e-9, "tilt_x": 0.0, "tilt_y": 0.0}
    ref = pref.ReferencePointCloudGPU()
    dst, (xyz, amp, cfg) = ref.run(pts, spec)
    torch.cuda.synchronize()
    ref_fringe = dst.cpu().numpy().astype(np.float64)

    def ref_call():
        dst.zero_()
        ref.launch(xyz, amp, cfg, dst)
    ref_ms = events_ms(ref_call, 2)
    p = PcParams(1.0, 1.0, 1.0, 0.0, 8e-6, 8e-6, nx, ny, 532e-9, 0.0, 0.0)
    tp = torch.from_numpy(pts).to(dev)
    out = {"workload": "point cloud 1024x1024, 5000 points (KETI exact r)", "reference_gpu_fp32_ms": ref_ms}
    fringes = {}
    for precision in ("fp64", "fp32"):
        cdt = torch.complex128 if precision == "fp64" else torch.complex64
        field = torch.empty((ny, nx), dtype=cdt, device=dev)
        fringe = torch.zeros((ny, nx), dtype=torch.float64 if precision == "fp64" else torch.float32, device=dev)

        def call():
            fringe.zero_()
            _lib.call("oh_pointcloud", ctx.handle, 1 if precision == "fp64" else 0, C.byref(p),
                      C.c_void_p(tp.data_ptr()), n, C.c_void_p(field.data_ptr()), C.c_void_p(fringe.data_ptr()), S())
        out[f"library_{precision}_ms"] = events_ms(call, 3)
        fringes[precision] = fringe.cpu().numpy().astype(np.float64)
    rel_ref, mx_ref = errs(ref_fringe, fringes["fp64"])
    rel32, mx32 = errs(fringes["fp32"], fringes["fp64"])
    out["reference_gpu_fp32_vs_library_fp64"] = {"rel": rel_ref, "max_abs_rel": mx_ref}
    out["library_fp32_vs_library_fp64"] = {"rel": rel32, "max_abs_rel": mx32}
    print(json.dumps(out))
    assert rel_ref < 0.1
    assert rel32 < 1e-4
