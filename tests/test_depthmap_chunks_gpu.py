"""Layer-chunked depth-map frames: with a small layer-buffer limit
(oh_ctx_set_depthmap_layer_limit) the row and column passes run per chunk of
layers and hand the spectrum accumulators on between chunks; the results
must equal the one-buffer frame bit for bit (the same operations in the
same order), and the layer buffer must stay within the limit."""
import numpy as np
import pytest
import torch

from openholo_gb300 import Context, _lib, depthmap as dm, scenes
from oracle import depthmap as odm

pytestmark = pytest.mark.gpu


def frame(ctx, p, img, depth, field=False):
    ti, td = torch.from_numpy(img).cuda(), torch.from_numpy(depth).cuda()
    f = torch.empty((p.pny, p.pnx), dtype=torch.complex64, device="cuda") if field else None
    fr = dm.generate(ctx, p, ti, td, field=f)
    torch.cuda.synchronize()
    return (fr.cpu().numpy(), f.cpu().numpy()) if field else fr.cpu().numpy()


@pytest.fixture
def chunked(lib_built):
    c = Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("kw", [dict(), dict(transform_viewing_window=1, field_lens=1.0)])
def test_chunked_frame_equals_single_buffer(ctx, chunked, kw):
    ny, nx, L = 540, 960, 12
    img, depth = scenes.depthmap_scene(17, ny, nx)
    p = dm.make_params(pnx=nx, pny=ny, num_of_depth=L, pad=2, phase_mode=dm.OH_PHASE_SEEDED, seed=5, **kw)
    ref = frame(ctx, p, img, depth)
    per_layer = ny * 2 * nx * 8
    _lib.call("oh_ctx_set_depthmap_layer_limit", chunked.handle, 2 * per_layer + 1)     # 6 chunks of 2 layers
    got = frame(chunked, p, img, depth)
    assert np.array_equal(got, ref)
    # the chunked context holds two layers' strips, not twelve
    assert _lib.lib().oh_ctx_scratch_bytes(chunked.handle) < (L // 2) * per_layer


def test_chunked_frame_with_empty_layers_between_chunks(ctx, chunked):
    """Layer-step gaps that cross chunk boundaries (levels 2, 3, 7, 8, 12 of 14
    used; chunks of 3 layers)."""
    ny, nx, L = 540, 960, 14
    img, depth0 = scenes.depthmap_scene(29, ny, nx)
    p = dm.make_params(pnx=nx, pny=ny, num_of_depth=L, pad=2, phase_mode=dm.OH_PHASE_SEEDED, seed=31)
    lut, _ = dm.levels(p)
    used = [2, 3, 7, 8, 12]
    byte_of = {lv: int(np.flatnonzero(lut == lv)[0]) for lv in used}
    band = (depth0.astype(np.int64) * len(used)) // 256
    depth = np.vectorize(lambda i: byte_of[used[i]])(band).astype(np.uint8)
    ref_fr, ref_f = frame(ctx, p, img, depth, field=True)
    _lib.call("oh_ctx_set_depthmap_layer_limit", chunked.handle, 3 * ny * 2 * nx * 8)
    fr, f = frame(chunked, p, img, depth, field=True)
    assert np.array_equal(fr, ref_fr) and np.array_equal(f, ref_f)
    op = odm.DMParams(pnx=nx, pny=ny, num_of_depth=L, pad=2)
    oracle_f = odm.generate(img, depth, op, phase=scenes.seeded_phase(31, ny, nx))[1]
    assert np.linalg.norm(f - oracle_f) / np.linalg.norm(oracle_f) < 2e-5


def test_full_size_frame_in_layer_chunks(ctx, chunked):
    """The 1920x1080, 32-layer benchmark frame with a 256 MiB layer buffer
    (about 4 layers per chunk instead of 1.06 GB for all 32)."""
    ny, nx = 1080, 1920
    img, depth = scenes.depthmap_scene(2024, ny, nx)
    p = dm.make_params(phase_mode=dm.OH_PHASE_SEEDED, seed=77)
    ref = frame(ctx, p, img, depth)
    _lib.call("oh_ctx_set_depthmap_layer_limit", chunked.handle, 256 << 20)
    got = frame(chunked, p, img, depth)
    assert np.array_equal(got, ref)
    assert _lib.lib().oh_ctx_scratch_bytes(chunked.handle) < 512 << 20


def test_chunked_batch_equals_single_buffer(ctx, chunked):
    frames_spec = [(512, 512, 9, 633e-9), (768, 768, 13, 532e-9), (384, 2048, 7, 450e-9)]
    out = []
    for c in (ctx, chunked):
        if c is chunked:
            _lib.call("oh_ctx_set_depthmap_layer_limit", chunked.handle, 3 * 512 * 1024 * 8)
        frames = []
        for i, (ny, nx, L, lam) in enumerate(frames_spec):
            img, depth = scenes.depthmap_scene(40 + i, ny, nx)
            p = dm.make_params(pnx=nx, pny=ny, num_of_depth=L, lam=lam, pad=2, phase_mode=dm.OH_PHASE_SEEDED,
                               seed=3 + i)
            frames.append((p, torch.from_numpy(img).cuda(), torch.from_numpy(depth).cuda(),
                           torch.empty((ny, nx), dtype=torch.float32, device="cuda")))
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            dm.generate_batch(c, frames, graph=True)
            dm.generate_batch(c, frames, graph=True)     # graph replay
        s.synchronize()
        out.append([f[3].cpu().numpy() for f in frames])
    for a, b in zip(*out):
        assert np.array_equal(a, b)
