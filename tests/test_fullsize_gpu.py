"""The benchmark configurations at their full sizes against the CPU oracle.

- 1920x1080 depth-map frame, 32 layers over 0.30-0.35 m, 2x zero pad, seeded
  per-pixel phase, FP32 (the headline workload): whole frame against
  oracle/depthmap.generate (HologramGenerator_CPU.cpp:117-270 restated).
- 1024x1024 point cloud, 5000 points (KETI exact r): FP64 <= 1e-9 and FP32
  <= 1e-3 against oracle_pc_f64 on seeded bands of rows.
- 200,000-point WRP, 64x64 windows, 3840x2160 at 3.74 um: against
  oracle_wrp_f64 (WRP.cpp:75-140 restated) on seeded 128x128 plane regions;
  the oracle runs every point whose window reaches a region, so the regions
  hold the complete sums.
- The 64-frame mixed batch in one call: three of its frames against the
  oracle.

Errors are reported as relative L2 and as max |error| / max |reference|.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, depthmap as dm, scenes
from openholo_gb300._lib import PcParams, WrpParams
from oracle import depthmap as odm
from oracle import pointcloud as opc

pytestmark = pytest.mark.gpu

TOL32 = 1e-3


def S():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def errs(got, ref):
    got = np.asarray(got, dtype=np.complex128 if np.iscomplexobj(got) else np.float64)
    ref = np.asarray(ref)
    d = got - ref
    return float(np.linalg.norm(d) / np.linalg.norm(ref)), float(np.abs(d).max() / np.abs(ref).max())


def oparams(p):
    return odm.DMParams(pnx=p.pnx, pny=p.pny, ppx=p.ppx, ppy=p.ppy, lam=p.lambda_, near=p.near_depthmap,
                        far=p.far_depthmap, num_of_depth=p.num_of_depth, pad=p.pad,
                        sig_location=(p.sig_location_x, p.sig_location_y))


def test_depthmap_1920x1080_L32_vs_oracle(ctx, dev):
    ny, nx = 1080, 1920
    img, depth = scenes.depthmap_scene(2024, ny, nx)
    p = dm.make_params(phase_mode=dm.OH_PHASE_SEEDED, seed=77)
    field = torch.empty((ny, nx), dtype=torch.complex64, device=dev)
    fr = dm.generate(ctx, p, torch.from_numpy(img).to(dev), torch.from_numpy(depth).to(dev), field=field)
    torch.cuda.synchronize()
    ref_fr, ref_field, _ = odm.generate(img, depth, oparams(p), phase=scenes.seeded_phase(77, ny, nx))
    rf, mf = errs(field.cpu().numpy(), ref_field)
    rr, mr = errs(fr.cpu().numpy(), ref_fr)
    print(f"1920x1080 L32 fp32: field rel {rf:.2e} max {mf:.2e}; fringe rel {rr:.2e} max {mr:.2e}")
    assert rf < TOL32 and rr < TOL32
    assert mf < TOL32 and mr < TOL32


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-3)])
def test_pointcloud_1024x1024_5000pts_vs_oracle(ctx, dev, precision, tol):
    n, nx, ny = 5000, 1024, 1024
    pts = scenes.pointcloud_scene(11, n).astype(np.float32)
    s = dict(scale_x=1.0, scale_y=1.0, scale_z=1.0, offset_depth=0.0, pitch_x=8e-6, pitch_y=8e-6, nx=nx, ny=ny,
             tilt_x=0.0, tilt_y=0.0)
    s["lambda"] = 532e-9
    p = PcParams(1.0, 1.0, 1.0, 0.0, 8e-6, 8e-6, nx, ny, 532e-9, 0.0, 0.0)
    tp = torch.from_numpy(pts).to(dev)
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    field = torch.empty((ny, nx), dtype=cdt, device=dev)
    _lib.call("oh_pointcloud", ctx.handle, 1 if precision == "fp64" else 0, C.byref(p), C.c_void_p(tp.data_ptr()),
              n, C.c_void_p(field.data_ptr()), None, S())
    torch.cuda.synchronize()
    got = field.cpu().numpy()
    rows = np.sort(np.random.default_rng(5).choice(ny - 8, 4, replace=False))
    for r0 in rows:                   # four bands of 8 rows, 41 M point-pixel terms in FP64
        ref = opc.pc_f64(pts.astype(np.float64), s, row0=int(r0), nrows=8)[r0:r0 + 8]
        rel, mx = errs(got[r0:r0 + 8], ref)
        print(f"pointcloud {precision} rows {r0}..{r0 + 7}: rel {rel:.2e} max {mx:.2e}")
        assert rel < tol and mx < 10 * tol


def test_wrp_200k_3840x2160_vs_oracle(ctx, dev):
    nx, ny, dp, lam, w = 3840, 2160, 3.74e-6, 532e-9, 32
    pts = scenes.wrp_scene(12, 200_000)
    z = float(pts[:, 2].min()) - 5e-3
    p = WrpParams(nx, ny, dp, lam, z, w)
    tp = torch.from_numpy(pts).to(dev)
    out = torch.zeros((ny, nx), dtype=torch.complex64, device=dev)
    _lib.call("oh_wrp_accumulate", ctx.handle, 0, C.byref(p), C.c_void_p(tp.data_ptr()), pts.shape[0],
              C.c_void_p(out.data_ptr()), S())
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    # window centres as the oracle places them (WRP.cpp:120-121, float pitch)
    tx = (pts[:, 0] / np.float64(np.float32(dp))).astype(np.int64) + nx // 2
    ty = (pts[:, 1] / np.float64(np.float32(dp))).astype(np.int64) + ny // 2
    rng = np.random.default_rng(3)
    occupied_x = (nx // 2 - 1200, nx // 2 + 1200 - 128)          # the 10 mm box spans ~2670 px
    occupied_y = (ny // 2 - 1000, ny // 2 + 1000 - 128)
    for _ in range(3):
        x0 = int(rng.integers(*occupied_x))
        y0 = int(rng.integers(*occupied_y))
        sel = (tx + w + 2 > x0) & (tx - w - 2 < x0 + 128) & (ty + w + 2 > y0) & (ty - w - 2 < y0 + 128)
        ref = opc.wrp_f64(pts[sel], nx, ny, dp, lam, z, w)[y0:y0 + 128, x0:x0 + 128]
        rel, mx = errs(got[y0:y0 + 128, x0:x0 + 128], ref)
        print(f"wrp region ({x0},{y0}) {int(sel.sum())} points: rel {rel:.2e} max {mx:.2e}")
        assert rel < 5e-5 and mx < 5e-4


def test_mixed_batch_frames_vs_oracle(ctx, dev):
    work = scenes.batch_workload()
    frames, scene = [], {}
    for i, (side, L, lam) in enumerate(work):
        if side not in scene:
            img, depth = scenes.depthmap_scene(scenes.BATCH_SCENE_SEED + side, side, side)
            scene[side] = (img, depth, torch.from_numpy(img).to(dev), torch.from_numpy(depth).to(dev))
        p = dm.make_params(pnx=side, pny=side, num_of_depth=L, lam=lam, pad=2, phase_mode=dm.OH_PHASE_SEEDED,
                           seed=scenes.BATCH_PHASE_SEED + i)
        frames.append((p, scene[side][2], scene[side][3],
                       torch.empty((side, side), dtype=torch.float32, device=dev)))
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        dm.generate_batch(ctx, frames, graph=True)
    s.synchronize()
    for i in (2, 27, 50):            # 768 px / 13 layers, 1536 / 14, 2048 / 12
        side, L, lam = work[i]
        p = frames[i][0]
        img, depth = scene[side][0], scene[side][1]
        ref = odm.generate(img, depth, oparams(p), phase=scenes.seeded_phase(scenes.BATCH_PHASE_SEED + i,
                                                                              side, side))[0]
        rel, mx = errs(frames[i][3].cpu().numpy(), ref)
        print(f"batch frame {i} ({side} px, {L} layers, {lam * 1e9:.0f} nm): rel {rel:.2e} max {mx:.2e}")
        assert rel < TOL32 and mx < TOL32
