"""oh_depthmap_generate_batch: frames of different sizes, layer counts and
wavelengths in one call, with and without CUDA-graph replay."""
import ctypes as C

import pytest
import torch

from openholo_gb300 import _lib, depthmap as dm, launch_count, scenes
from openholo_gb300._lib import OhError

pytestmark = pytest.mark.gpu

# (pny, pnx, layers, wavelength): scheduled FFT lengths (1024, 1536, 1080x1920,
# and padded length 4096 along x and along y, whose shared-memory lines carry
# the per-radix pads) and a generic one (192 x 240)
FRAMES = [(512, 512, 6, 633e-9), (96, 120, 5, 450e-9), (768, 768, 9, 532e-9), (540, 960, 4, 450e-9),
          (384, 2048, 3, 532e-9), (2048, 384, 3, 633e-9)]


def _frames(seed):
    out = []
    for i, (ny, nx, L, lam) in enumerate(FRAMES):
        img, depth = scenes.depthmap_scene(seed + i, ny, nx)
        p = dm.make_params(pnx=nx, pny=ny, num_of_depth=L, lam=lam, pad=2, phase_mode=dm.OH_PHASE_SEEDED,
                           seed=77 + i)
        out.append((p, torch.from_numpy(img).cuda(), torch.from_numpy(depth).cuda(),
                    torch.empty((ny, nx), dtype=torch.float32, device="cuda")))
    return out


def test_batch_equals_single_frames(ctx):
    frames = _frames(10)
    dm.generate_batch(ctx, frames)
    torch.cuda.synchronize()
    for p, img, depth, fr in frames:
        ref = dm.generate(ctx, p, img, depth)
        torch.cuda.synchronize()
        assert torch.equal(fr, ref)


def test_batch_graph_replays_on_new_inputs(ctx):
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        frames = _frames(20)
        dm.generate_batch(ctx, frames, graph=True)          # runs the frames and captures them
        first = [f[3].clone() for f in frames]
        for f in frames:
            f[3].zero_()
        n0 = launch_count()
        dm.generate_batch(ctx, frames, graph=True)          # graph replay
        assert launch_count() - n0 >= 3 * len(frames)
        for f, a in zip(frames, first):
            assert torch.equal(f[3], a)
        # new scene content in the same buffers: the replay reads it
        for i, (ny, nx, _, _) in enumerate(FRAMES):
            img, depth = scenes.depthmap_scene(90 + i, ny, nx)
            frames[i][1].copy_(torch.from_numpy(img).cuda())
            frames[i][2].copy_(torch.from_numpy(depth).cuda())
        dm.generate_batch(ctx, frames, graph=True)
        got = [f[3].clone() for f in frames]
        # a single frame with other parameters between replays must not disturb them
        dm.generate(ctx, dm.make_params(pnx=64, pny=48, num_of_depth=3), frames[1][1][:48, :64].contiguous(),
                    frames[1][2][:48, :64].contiguous())
        for (p, img, depth, fr), g in zip(frames, got):
            ref = dm.generate(ctx, p, img, depth)
            assert torch.equal(g, ref)
        dm.generate_batch(ctx, frames, graph=True)
        for f, g in zip(frames, got):
            assert torch.equal(f[3], g)
    s.synchronize()


def test_batch_arguments(ctx):
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("oh_depthmap_generate_batch", ctx.handle, 0, None, 0, 0, st)      # empty batch
    arr = (_lib.DepthmapFrame * 1)()
    arr[0].params = dm.make_params(pnx=64, pny=48, num_of_depth=3)
    with pytest.raises(OhError):            # missing buffers
        _lib.call("oh_depthmap_generate_batch", ctx.handle, 0, arr, 1, 0, st)
    with pytest.raises(OhError):            # unknown flag
        _lib.call("oh_depthmap_generate_batch", ctx.handle, 0, arr, 1, 8, st)
