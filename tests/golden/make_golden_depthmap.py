"""Generate tests/golden/dm_reference_gpu.npz from the reference's own
depth-map GPU kernels.

Needs a CUDA GPU and oracle/_ref/dm_ref.cubin, which oracle/build.py compiles
from the reference's OpenHolo_DepthMap/Hologram/src/HologramKernel.cu in a
checkout that has the reference tree; the cubin then travels with the
checkout.  oracle/dm_reference.py issues the kernels in the reference's call
sequence (Calc_Holo_GPU, encoding_GPU).  Run:

    python tests/golden/make_golden_depthmap.py [output.npz]

Each case stores its parameters (JSON), the seeded uint8 image and depth map,
the reference's u255 fringe (float64) and, where marked, the accumulated
angular spectrum u_complex before encoding (complex128).
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import depthmap as odm  # noqa: E402

OUT = Path(__file__).resolve().parent / "dm_reference_gpu.npz"

# name -> (params, image seed, store spectrum)
CASES = {
    # 8 um, 532 nm, 16 levels over 0.30-0.34 m (near/far chosen, here and below,
    # so that GetDepthValues' accumulation loop yields all num_of_depth levels)
    "a": (dict(pnx=256, pny=128, ppx=8e-6, ppy=8e-6, lam=532e-9, field_lens=1.0, near=0.30, far=0.34,
               num_of_depth=16, flag_change_depth_quantization=1, transform_viewing_window=1,
               sig_location=(0, 1)), 11, False),
    # FLAG_CHANGE_DEPTH_QUANTIZATION = 0: layer = 256 - depth byte, all 256 levels;
    # the sample configuration's pitch, wavelength and field lens; constant
    # non-trivial rand_phase; signal in the lower-right quadrant
    "b": (dict(pnx=192, pny=128, ppx=12.7e-6 / 3, ppy=12.7e-6, lam=633e-9, field_lens=0.5, near=0.15, far=0.45,
               num_of_depth=256, flag_change_depth_quantization=0, default_depth_quantization=256,
               transform_viewing_window=1, sig_location=(1, -1), rand_phase=complex(np.cos(0.7), np.sin(0.7))),
          12, False),
    # a render_depth subset, both signal offsets negative
    "c": (dict(pnx=128, pny=128, ppx=6.4e-6, ppy=6.4e-6, lam=473e-9, field_lens=1.0, near=0.12, far=0.20,
               num_of_depth=8, flag_change_depth_quantization=1, transform_viewing_window=1,
               sig_location=(-1, -1), render_depth=[2, 3, 5, 8]), 13, True),
    # odd frame sizes (fftShift by floor(n/2) on both sides)
    "d": (dict(pnx=121, pny=77, ppx=8e-6, ppy=8e-6, lam=532e-9, field_lens=1.0, near=0.30, far=0.34,
               num_of_depth=5, flag_change_depth_quantization=1, transform_viewing_window=1,
               sig_location=(0, 1)), 14, True),
}


def make_inputs(seed: int, ny: int, nx: int):
    """Smooth seeded image and depth map (uint8); about 15 % of the image
    pixels are zero so that the alpha map (img > 0) matters."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:ny, 0:nx] / max(nx, ny)
    img = np.zeros((ny, nx))
    dep = np.zeros((ny, nx))
    for _ in range(6):
        cx, cy, s = rng.uniform(0, 1), rng.uniform(0, 1), rng.uniform(0.05, 0.3)
        img += rng.uniform(0.3, 1.0) * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s))
        cx, cy, s = rng.uniform(0, 1), rng.uniform(0, 1), rng.uniform(0.2, 0.6)
        dep += rng.uniform(0.3, 1.0) * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s))
    img = np.rint(255 * img / img.max()).astype(np.uint8)
    img[rng.random((ny, nx)) < 0.15] = 0
    dep = np.rint(255 * (dep - dep.min()) / (dep.max() - dep.min())).astype(np.uint8)
    return img, dep


def params(d: dict) -> odm.DMParams:
    d = dict(d)
    d["sig_location"] = tuple(d["sig_location"])
    if "rand_phase" in d:
        d["rand_phase"] = complex(*d["rand_phase"]) if isinstance(d["rand_phase"], list) else d["rand_phase"]
    return odm.DMParams(pad=1, **d)


def raw_level_count(p: odm.DMParams) -> int:
    """Number of levels GetDepthValues' accumulation loop produces
    (HologramGenerator.cpp:393-402); the reference reads dlevel_[0..nd-1]."""
    dstep = (p.far - p.near) / (p.num_of_depth - 1)
    n, val = 0, p.near
    while val <= p.far:
        n += 1
        val += dstep
    return n


def main():
    from oracle.dm_reference import ReferenceGPU
    out = Path(sys.argv[1]) if len(sys.argv) > 1 else OUT
    arrays, meta = {}, {}
    for name, (d, seed, keep_spec) in CASES.items():
        p = params(d)
        assert raw_level_count(p) >= p.num_of_depth, name
        img, dep = make_inputs(seed, p.pny, p.pnx)
        fringe, spec = ReferenceGPU(p).generate(img, dep)
        arrays[f"{name}_img"] = img
        arrays[f"{name}_depth"] = dep
        arrays[f"{name}_fringe"] = fringe
        if keep_spec:
            arrays[f"{name}_spectrum"] = spec
        dj = dict(d)
        if "rand_phase" in dj:
            dj["rand_phase"] = [dj["rand_phase"].real, dj["rand_phase"].imag]
        meta[name] = dict(params=dj, seed=seed)
        ref = odm.generate(img, dep, p)[0]
        err = np.abs(fringe - ref).max() / np.abs(ref).max()
        print(f"case {name}: {p.pnx}x{p.pny}, {p.num_of_depth} levels: oracle vs reference kernels max {err:.2e}")
    np.savez_compressed(out, cases=json.dumps(meta), **arrays)
    print("wrote", out)


if __name__ == "__main__":
    main()
