"""The seeded synthetic workloads (no GPU): the mixed depth-map batch draws
its frames from the stated sets and is reproducible; the scenes are uint8
frames of the requested shape with both intensity and depth spanning their
range."""
import numpy as np

from openholo_gb300 import scenes


def test_batch_workload_distribution_and_determinism():
    work = scenes.batch_workload()
    assert len(work) == 64
    assert work == scenes.batch_workload()                       # same seed, same batch
    assert scenes.batch_workload(seed=scenes.BATCH_SEED + 1) != work
    sides = {s for s, _, _ in work}
    assert sides <= {512, 768, 1024, 1536, 2048} and len(sides) == 5
    assert all(8 <= L <= 64 for _, L, _ in work)
    assert {lam for _, _, lam in work} == {450e-9, 532e-9, 633e-9}


def test_depthmap_scene_shape_and_range():
    img, depth = scenes.depthmap_scene(7, 96, 160)
    assert img.shape == depth.shape == (96, 160)
    assert img.dtype == depth.dtype == np.uint8
    assert img.max() == 255 and depth.min() == 0 and depth.max() == 255
    i2, d2 = scenes.depthmap_scene(7, 96, 160)
    assert np.array_equal(img, i2) and np.array_equal(depth, d2)


def test_seeded_phase_is_uniform_in_turns():
    ph = scenes.seeded_phase(3, 64, 64)
    assert ph.shape == (64, 64)
    assert ph.min() >= 0.0 and ph.max() < 2 * np.pi
    assert abs(ph.mean() - np.pi) < 0.1
