"""The depth-map path against golden fixtures produced by the reference's own
GPU kernels (tests/golden/dm_reference_gpu.npz, written by
tests/golden/make_golden_depthmap.py: HologramKernel.cu compiled from the
reference's source and issued in the order of Calc_Holo_GPU / encoding_GPU,
with cuFFT Z2Z).

- CPU: the float64 oracle (oracle/depthmap.py) reproduces every fixture to
  FP64 rounding (measured 4e-16 to 6e-16 relative; bound 1e-13 relative L2
  and max |error| / max |fringe|).
- GPU: the library's FP64 mode (pad 1, constant reference phase) to 1e-7
  relative (measured 5e-11 to 1.4e-10), and its FP32 mode to 1e-3 (measured
  2e-7 to 4e-7), against the same fixtures.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import depthmap as odm

FIX = Path(__file__).resolve().parent / "golden" / "dm_reference_gpu.npz"


def load():
    z = np.load(FIX)
    cases = json.loads(str(z["cases"]))
    return z, cases


def oparams(d):
    d = dict(d)
    d["sig_location"] = tuple(d["sig_location"])
    if "rand_phase" in d:
        d["rand_phase"] = complex(*d["rand_phase"])
    return odm.DMParams(pad=1, **d)


def errs(got, ref):
    d = np.asarray(got) - ref
    return float(np.linalg.norm(d) / np.linalg.norm(ref)), float(np.abs(d).max() / np.abs(ref).max())


CASE_NAMES = ["a", "b", "c", "d"]


@pytest.mark.parametrize("name", CASE_NAMES)
def test_oracle_matches_reference_kernels(name):
    z, cases = load()
    p = oparams(cases[name]["params"])
    img, dep = z[f"{name}_img"], z[f"{name}_depth"]
    fr, _, U = odm.generate(img, dep, p)
    rel, mx = errs(fr, z[f"{name}_fringe"])
    print(f"case {name}: fringe rel {rel:.2e} max {mx:.2e}")
    assert rel < 1e-13 and mx < 1e-13
    if f"{name}_spectrum" in z:
        rel, mx = errs(U, z[f"{name}_spectrum"])
        print(f"case {name}: spectrum rel {rel:.2e} max {mx:.2e}")
        assert rel < 1e-13 and mx < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-7), ("fp32", 1e-3)])
@pytest.mark.parametrize("name", CASE_NAMES)
def test_library_matches_reference_kernels(ctx, dev, name, precision, tol):
    import torch
    from openholo_gb300 import depthmap as dm
    z, cases = load()
    d = cases[name]["params"]
    p = dm.make_params(pnx=d["pnx"], pny=d["pny"], ppx=d["ppx"], ppy=d["ppy"], lam=d["lam"], near=d["near"],
                       far=d["far"], num_of_depth=d["num_of_depth"],
                       flag_change_depth_quantization=d["flag_change_depth_quantization"],
                       default_depth_quantization=d.get("default_depth_quantization", 256),
                       transform_viewing_window=d["transform_viewing_window"], field_lens=d["field_lens"], pad=1,
                       sig_location=tuple(d["sig_location"]), phase_mode=dm.OH_PHASE_REFERENCE,
                       rand_phase=complex(*d.get("rand_phase", [1.0, 0.0])), render_depth=d.get("render_depth"))
    img = torch.from_numpy(z[f"{name}_img"]).to(dev)
    dep = torch.from_numpy(z[f"{name}_depth"]).to(dev)
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    spec = torch.empty((p.pny, p.pnx), dtype=cdt, device=dev)
    fr = dm.generate(ctx, p, img, dep, precision=precision, spectrum=spec)
    torch.cuda.synchronize()
    rel, mx = errs(fr.cpu().numpy().astype(np.float64), z[f"{name}_fringe"])
    print(f"case {name} {precision}: fringe rel {rel:.2e} max {mx:.2e}")
    assert rel < tol and mx < 10 * tol
    if f"{name}_spectrum" in z:
        rel, _ = errs(spec.cpu().numpy().astype(np.complex128), z[f"{name}_spectrum"])
        print(f"case {name} {precision}: spectrum rel {rel:.2e}")
        assert rel < tol
