"""The persistent depth-map batch kernel: every frame of a batch in one launch
(work items taken from a device queue, bounded waits on the passes they read
from).  Its frames must equal the per-frame path's bit for bit (the same
pass bodies run with 256 threads), and the per-frame path is checked against
the oracle elsewhere; two frames here are also checked against the oracle
directly.  The reference generates one frame per call
(OpenHolo_DepthMap/Hologram/src/HologramGenerator.cpp:261-294)."""
import ctypes as C

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, depthmap as dm, launch_count, scenes
from oracle import depthmap as odm

pytestmark = pytest.mark.gpu

TIMEOUT = 5
# (pny, pnx, layers, wavelength): every padded length the batch kernel
# carries (1024 .. 4096), square and not, along both axes
FRAMES = [(512, 512, 8, 633e-9), (768, 768, 13, 532e-9), (1024, 1024, 9, 450e-9), (512, 2048, 6, 532e-9),
          (2048, 512, 7, 450e-9), (1536, 1536, 5, 633e-9), (1024, 768, 11, 532e-9), (512, 512, 3, 450e-9)]


def _frames(seed, spec=FRAMES):
    out = []
    for i, (ny, nx, L, lam) in enumerate(spec):
        img, depth = scenes.depthmap_scene(seed + i, ny, nx)
        p = dm.make_params(pnx=nx, pny=ny, num_of_depth=L, lam=lam, pad=2, phase_mode=dm.OH_PHASE_SEEDED,
                           seed=300 + i)
        out.append((p, torch.from_numpy(img).cuda(), torch.from_numpy(depth).cuda(),
                    torch.empty((ny, nx), dtype=torch.float32, device="cuda")))
    return out


def _mode(ctx, persistent):
    dm.set_batch_mode(ctx, bool(persistent))


def S():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_persistent_batch_equals_per_frame(ctx):
    frames = _frames(40)
    _mode(ctx, 1)
    dm.generate_batch(ctx, frames)                 # builds the plan: set-up + batch kernel
    n0 = launch_count()
    dm.generate_batch(ctx, frames)
    torch.cuda.synchronize()
    assert launch_count() - n0 == 1                # one launch for the whole batch
    for p, img, depth, fr in frames:
        ref = dm.generate(ctx, p, img, depth)
        torch.cuda.synchronize()
        assert torch.equal(fr, ref)


def test_persistent_batch_vs_oracle(ctx):
    spec = [(512, 512, 6, 532e-9), (768, 512, 5, 633e-9)]
    frames = _frames(60, spec)
    _mode(ctx, 1)
    dm.generate_batch(ctx, frames)
    torch.cuda.synchronize()
    for i, ((ny, nx, L, lam), (p, img, depth, fr)) in enumerate(zip(spec, frames)):
        op = odm.DMParams(pnx=nx, pny=ny, num_of_depth=L, pad=2, lam=lam)
        phase = scenes.seeded_phase(300 + i, ny, nx)
        ref, _, _ = odm.generate(img.cpu().numpy(), depth.cpu().numpy(), op, phase=phase)
        got = fr.cpu().numpy().astype(np.float64)
        rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert rel < 1e-4, rel


def test_persistent_graph_replays_on_new_inputs(ctx):
    _mode(ctx, 1)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        frames = _frames(70)
        dm.generate_batch(ctx, frames, graph=True)          # plan, then capture and launch the graph
        first = [f[3].clone() for f in frames]
        for f in frames:
            f[3].zero_()
        n0 = launch_count()
        dm.generate_batch(ctx, frames, graph=True)          # graph replay: one kernel
        assert launch_count() - n0 == 1
        for f, a in zip(frames, first):
            assert torch.equal(f[3], a)
        for i, (ny, nx, _, _) in enumerate(FRAMES):
            img, depth = scenes.depthmap_scene(170 + i, ny, nx)
            frames[i][1].copy_(torch.from_numpy(img).cuda())
            frames[i][2].copy_(torch.from_numpy(depth).cuda())
        dm.generate_batch(ctx, frames, graph=True)
        got = [f[3].clone() for f in frames]
        for (p, img, depth, fr), g in zip(frames, got):
            assert torch.equal(g, dm.generate(ctx, p, img, depth))
    s.synchronize()


def test_batch_modes_agree_and_fallback(ctx):
    # a frame the batch kernel does not carry (1080x1920: padded 2160 x 3840)
    # sends the whole batch through the per-frame launches
    spec = FRAMES[:3] + [(540, 960, 4, 450e-9)]
    frames = _frames(80, spec)
    _mode(ctx, 1)
    n0 = launch_count()
    dm.generate_batch(ctx, frames)
    torch.cuda.synchronize()
    assert launch_count() - n0 >= 3 * len(spec)
    a = [f[3].clone() for f in frames]
    frames = _frames(80, FRAMES)
    _mode(ctx, 0)
    dm.generate_batch(ctx, frames)
    torch.cuda.synchronize()
    per = [f[3].clone() for f in frames]
    _mode(ctx, 1)
    dm.generate_batch(ctx, frames)
    torch.cuda.synchronize()
    for f, b in zip(frames, per):
        assert torch.equal(f[3], b)
    for (p, img, depth, fr), g in zip(_frames(80, spec), a):
        assert torch.equal(g, dm.generate(ctx, p, img, depth))


def test_persistent_batch_wait_runs_out(ctx):
    frames = _frames(90, FRAMES[:4])
    _mode(ctx, 1)
    assert _lib.lib().oh_ctx_device_status(ctx.handle, S()) == 0
    _lib.call("oh_ctx_set_test_stall", ctx.handle, 8, 2_000_000)
    try:
        dm.generate_batch(ctx, frames)
        assert _lib.lib().oh_ctx_device_status(ctx.handle, S()) == TIMEOUT
    finally:
        _lib.call("oh_ctx_set_test_stall", ctx.handle, 0, 0)
    dm.generate_batch(ctx, frames)
    assert _lib.lib().oh_ctx_device_status(ctx.handle, S()) == 0
    for p, img, depth, fr in frames:
        assert torch.equal(fr, dm.generate(ctx, p, img, depth))


def test_autotune_batch(ctx, tmp_path):
    # two frames of each of two lengths; the tune file keeps the entries
    spec = [(512, 512, 6, 532e-9), (512, 512, 9, 633e-9), (768, 768, 5, 450e-9), (768, 768, 7, 532e-9),
            (512, 2048, 4, 532e-9)]
    frames = _frames(110, spec)
    path = tmp_path / "tune.txt"
    dm.set_autotune_file(ctx, path)
    dm.set_batch_mode(ctx, True)
    dm.autotune_batch(ctx, frames, reps=1)
    torch.cuda.synchronize()
    lines = [l.split() for l in path.read_text().splitlines() if not l.startswith("#")]
    keys = {l[0].rsplit(":", 1)[1] for l in lines}
    assert {"1024", "1536"} <= keys
    for L in (1024, 1536):
        t = dm.batch_tuning(ctx, L)
        assert t["ctas_per_sm"] in (1, 2) and t["lag"] in (0, 1) and t["col_w"] in (1, 2)
        assert t["row_pairs"] in (1, 2, 4) and t["col_blocks"] in (1, 2) and t["out_rows"] in (1, 2, 4, 8)
        assert t["ms"] > 0
    # a batch after tuning still equals the per-frame path
    n0 = launch_count()
    dm.generate_batch(ctx, frames)
    torch.cuda.synchronize()
    assert launch_count() - n0 == 2                # table set-up + batch kernel (new plan)
    for p, img, depth, fr in frames:
        assert torch.equal(fr, dm.generate(ctx, p, img, depth))
    # another context reads the same settings from the file
    other = _lib.Context(0)
    dm.set_autotune_file(other, path)
    try:
        for L in (1024, 1536):
            a, b = dm.batch_tuning(other, L), dm.batch_tuning(ctx, L)
            assert a.pop("ms") == pytest.approx(b.pop("ms"), rel=1e-5)
            assert a == b
    finally:
        other.close()
    dm.set_autotune_file(ctx, None)


def test_persistent_batch_phase_arrays_and_fields(ctx):
    # per-pixel phase arrays and complex field outputs through the batch kernel
    spec = [(512, 512, 7, 532e-9), (768, 512, 5, 450e-9), (1024, 1024, 4, 633e-9)]
    frames, ref_inputs = [], []
    for i, (ny, nx, L, lam) in enumerate(spec):
        img, depth = scenes.depthmap_scene(120 + i, ny, nx)
        phase = torch.from_numpy(scenes.seeded_phase(500 + i, ny, nx).astype(np.float32)).cuda()
        p = dm.make_params(pnx=nx, pny=ny, num_of_depth=L, lam=lam, pad=2, phase_mode=dm.OH_PHASE_ARRAY)
        ti, td = torch.from_numpy(img).cuda(), torch.from_numpy(depth).cuda()
        fr = torch.empty((ny, nx), dtype=torch.float32, device="cuda")
        fd = torch.empty((ny, nx), dtype=torch.complex64, device="cuda")
        frames.append((p, ti, td, fr, phase, fd))
    _mode(ctx, 1)
    n0 = launch_count()
    dm.generate_batch(ctx, frames)
    torch.cuda.synchronize()
    assert launch_count() - n0 == 2                        # table set-up + batch kernel
    for p, ti, td, fr, phase, fd in frames:
        rf = torch.empty_like(fd)
        ref = dm.generate(ctx, p, ti, td, phase=phase, field=rf)
        torch.cuda.synchronize()
        assert torch.equal(fr, ref)
        assert torch.equal(fd, rf)


def test_persistent_batch_of_one_frame(ctx):
    frames = _frames(130, [(1024, 1024, 16, 532e-9)])
    _mode(ctx, 1)
    dm.generate_batch(ctx, frames)
    n0 = launch_count()
    dm.generate_batch(ctx, frames)
    torch.cuda.synchronize()
    assert launch_count() - n0 == 1
    p, img, depth, fr = frames[0]
    assert torch.equal(fr, dm.generate(ctx, p, img, depth))


def test_tune_file_errors(ctx, tmp_path):
    bad = tmp_path / "bad.txt"
    bad.write_text("# header\nsm_103:152:1024 2 1 2 1\n")        # too few fields
    with pytest.raises(_lib.OhError):
        dm.set_autotune_file(ctx, bad)
    bad.write_text("sm_103:152:1024 3 1 2 1 1 2 1.0\n")            # 3 blocks per SM is not a setting
    with pytest.raises(_lib.OhError):
        dm.set_autotune_file(ctx, bad)
    dm.set_autotune_file(ctx, tmp_path / "absent.txt")              # created by the first autotune
    dm.set_autotune_file(ctx, None)


def _tune_key(length):
    maj, mnr = torch.cuda.get_device_capability(0)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    return f"sm_{maj}{mnr}:{sms}:{length}"


@pytest.mark.parametrize("ctas,lag,col_w,row_pairs,col_blocks,out_rows", [
    (1, 0, 1, 4, 2, 8), (2, 0, 2, 2, 1, 1), (1, 1, 1, 1, 2, 4), (2, 1, 1, 4, 2, 1)])
def test_persistent_batch_settings_keep_results(ctx, tmp_path, ctas, lag, col_w, row_pairs, col_blocks, out_rows):
    # every setting the tuner can pick gives the per-frame results bit for bit
    # (settings given through a tune file for the lengths of these frames)
    spec = [(512, 512, 9, 532e-9), (768, 768, 6, 633e-9), (512, 512, 13, 450e-9), (768, 512, 5, 532e-9)]
    path = tmp_path / "tune.txt"
    lines = [f"{_tune_key(n)} {ctas} {lag} {col_w} {row_pairs} {col_blocks} {out_rows} 0.0" for n in (1024, 1536)]
    path.write_text("\n".join(lines) + "\n")
    dm.set_autotune_file(ctx, path)
    try:
        for L in (1024, 1536):
            t = dm.batch_tuning(ctx, L)
            assert (t["ctas_per_sm"], t["lag"], t["col_w"], t["row_pairs"], t["col_blocks"], t["out_rows"]) == \
                (ctas, lag, col_w, row_pairs, col_blocks, out_rows)
        frames = _frames(140, spec)
        _mode(ctx, 1)
        dm.generate_batch(ctx, frames)
        torch.cuda.synchronize()
        for p, img, depth, fr in frames:
            assert torch.equal(fr, dm.generate(ctx, p, img, depth))
    finally:
        dm.set_autotune_file(ctx, None)
