"""The learned surrogate's pipeline on the GPU: the seeded RGB-D scene
generator against its float64 twin, the complex-source propagation against
the layered frame and the oracle, the mid-plane decomposition of the plain
method, and the PSNR-gated fallback."""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import depthmap as dm, scenes, surrogate
from oracle import depthmap as odm

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_scene_generator_matches_float64_twin(ctx):
    n, h, w = 3, 96, 160
    got = surrogate.scenes_rgbd(ctx, 40, n, h, w).cpu().numpy()
    for f in range(n):
        ref = scenes.rgbd_scene(40 + f, h, w)
        d = np.abs(got[f].astype(np.int32) - ref.astype(np.int32))
        assert d.max() <= 1 and np.count_nonzero(d) <= 2e-3 * d.size
    # G and depth are the depth-map scene of the same seed
    img, depth = scenes.depthmap_scene(40, h, w)
    assert np.abs(got[0][..., 1].astype(int) - img.astype(int)).max() <= 1


def test_complex_source_equals_single_layer_frame(ctx):
    """A flat-depth frame is one layer: its source field img/255 exp(i phase)
    through oh_depthmap_propagate_field at that layer's z' gives the frame."""
    ny, nx = 128, 256
    img, _ = scenes.depthmap_scene(3, ny, nx)
    depth = np.full((ny, nx), 100, np.uint8)
    phase = scenes.seeded_phase(8, ny, nx)
    p = dm.make_params(pnx=nx, pny=ny, num_of_depth=16, pad=2, phase_mode=dm.OH_PHASE_ARRAY)
    lut, z = dm.levels(p)
    zl = float(z[lut[100] - 1])
    ref_fr = dm.generate(ctx, p, torch.from_numpy(img).cuda(), torch.from_numpy(depth).cuda(),
                         torch.from_numpy(phase).cuda())
    src = torch.from_numpy((img / 255.0 * np.exp(1j * phase.astype(np.float64))).astype(np.complex64)).cuda()
    fr = dm.propagate_field(ctx, p, src, zl)
    torch.cuda.synchronize()
    assert rel(fr.cpu().numpy(), ref_fr.cpu().numpy()) < 1e-5
    op = odm.DMParams(pnx=nx, pny=ny, num_of_depth=16, pad=2)
    oracle_fr = odm.generate(img, depth, op, phase=phase)[0]
    assert rel(fr.cpu().numpy(), oracle_fr) < 1e-3


def test_mid_plane_decomposition(ctx):
    """Plain layers -> mid plane (levels shifted by -z_mid, full spectrum) ->
    hologram over z_mid equals the direct frame, for a scene away from the
    frame edges (the mid-plane field is kept on the frame, so light that
    leaves it is lost)."""
    h = w = 256
    rgbd = surrogate.scenes_rgbd(ctx, 11, 1, h, w)[0]
    r = rgbd.cpu().numpy().copy()
    r[:64], r[-64:], r[:, :64], r[:, -64:] = 0, 0, 0, 0
    rgbd = torch.from_numpy(r).cuda()
    p = dm.make_params(pnx=w, pny=h, num_of_depth=32, pad=2)
    z_mid = 0.325
    F = surrogate.mid_field(ctx, p, z_mid, rgbd)
    two_step = dm.propagate_field(ctx, p, F, z_mid)
    direct = dm.generate(ctx, p, rgbd[..., 1].contiguous(), rgbd[..., 3].contiguous())
    torch.cuda.synchronize()
    err = rel(two_step.cpu().numpy(), direct.cpu().numpy())
    print("two-step vs direct:", err)
    assert err < 2e-2


def test_fallback_replaces_a_poor_prediction(ctx):
    h = w = 128
    net = surrogate.UNet(ctx, max_batch=1, max_height=h, max_width=w, seed=3, out_scale=1.0)
    try:
        rgbd = surrogate.scenes_rgbd(ctx, 5, 1, h, w)[0]
        p = dm.make_params(pnx=w, pny=h, num_of_depth=32, pad=2)
        z_mid = 0.325
        F = surrogate.mid_field(ctx, p, z_mid, rgbd)
        plain_fr = dm.propagate_field(ctx, p, F, z_mid)
        pred = net.forward(rgbd[None])[0]
        pred_fr = dm.propagate_field(ctx, p, pred, z_mid)
        # untrained: far below 40 dB, the plain field is used
        fr, rep = surrogate.generate(ctx, net, p, z_mid, rgbd, check=True, psnr_threshold_db=40.0)
        torch.cuda.synchronize()
        assert rep["checked"] == 1 and rep["fell_back"] == 1 and rep["psnr_db"] < 40.0
        assert torch.equal(fr, plain_fr)
        # a threshold the prediction passes keeps it
        fr2, rep2 = surrogate.generate(ctx, net, p, z_mid, rgbd, check=True, psnr_threshold_db=-1e9)
        assert rep2["fell_back"] == 0 and torch.equal(fr2, pred_fr)
        # no check: the prediction, no report
        fr3, rep3 = surrogate.generate(ctx, net, p, z_mid, rgbd, check=False)
        torch.cuda.synchronize()
        assert rep3["checked"] == 0 and torch.equal(fr3, pred_fr)
        # the reported errors against the plain field
        a, b = pred.cpu().numpy().astype(np.complex128), F.cpu().numpy().astype(np.complex128)
        assert rep["rel_err"] == pytest.approx(rel(a, b), rel=1e-3)
        ib, ia = np.abs(b) ** 2, np.abs(a) ** 2
        psnr = 10 * np.log10(ib.max() ** 2 / np.mean((ia - ib) ** 2))
        assert rep["psnr_db"] == pytest.approx(psnr, abs=1e-2)
    finally:
        net.close()


def test_training_gains_over_the_untrained_network(ctx):
    """Training on the GPU against the plain method's mid-plane fields (256 x
    256 frames, 1600 samples) lifts the held-out PSNR well above the untrained
    network's (measured 17.6 -> 25.8 dB); the gate's decision follows the
    PSNR."""
    h = w = 256
    p = dm.make_params(pnx=w, pny=h, num_of_depth=32, pad=2)
    lut, _ = dm.levels(p)
    dl = np.where(lut > 0, (lut - 1) / 31.0, 0.0).astype(np.float32)
    z_mid = 0.325
    probe = surrogate.scenes_rgbd(ctx, 77, 1, h, w)[0]
    rms = float(torch.sqrt((surrogate.mid_field(ctx, p, z_mid, probe).abs() ** 2).mean()))
    net = surrogate.UNet(ctx, max_batch=4, max_height=h, max_width=w, seed=2, out_scale=rms, depth_lut=dl)
    try:
        held = [surrogate.scenes_rgbd(ctx, 5000 + i, 1, h, w)[0] for i in range(4)]

        def psnrs(threshold=40.0):
            return [surrogate.generate(ctx, net, p, z_mid, r, check=True, psnr_threshold_db=threshold)[1]
                    for r in held]
        before = psnrs()
        losses = surrogate.train(ctx, net, p, z_mid, samples=1600, batch=4, lr=1e-3, seed=100)
        after = psnrs()
        b = np.mean([r["psnr_db"] for r in before])
        a = np.mean([r["psnr_db"] for r in after])
        print(f"held-out mid-plane PSNR: untrained {b:.1f} dB, trained {a:.1f} dB; "
              f"loss {np.mean(losses[:10]):.3e} -> {np.mean(losses[-10:]):.3e}")
        assert a > b + 5.0
        assert np.mean(losses[-10:]) < 0.2 * np.mean(losses[:10])
        # the gate: a threshold below every trained PSNR keeps every prediction
        keep = psnrs(threshold=min(r["psnr_db"] for r in after) - 1.0)
        assert sum(r["fell_back"] for r in keep) == 0
        assert all(r["fell_back"] == (r["psnr_db"] < 40.0) for r in after)
    finally:
        net.close()
