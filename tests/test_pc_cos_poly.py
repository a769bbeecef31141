"""The point-cloud kernel's cosine polynomial (pc_sincos2 in pointcloud.cu):
its coefficients, read from the source, evaluated by FP32 Horner steps on a
dense grid over [-pi, pi], stay within the error bound the source states."""
import re
from pathlib import Path

import numpy as np

SRC = Path(__file__).resolve().parents[1] / "openholo_gb300" / "csrc" / "pointcloud.cu"


def _coefficients():
    body = SRC.read_text()
    body = body[body.index("void pc_sincos2"):]
    body = body[:body.index("\n}\n")]
    vals = re.findall(r"make_float2\(([-+0-9.eE]+)f, \1f\)", body)
    return [np.float32(v) for v in vals]


def test_cos_polynomial_error_bound():
    c = _coefficients()          # Horner order: highest power first, then the +1
    assert len(c) == 7
    x = np.linspace(-np.pi, np.pi, 400001).astype(np.float32)
    t = (x * x).astype(np.float32)
    q = np.full_like(t, c[0])
    for ci in c[1:]:
        # one FMA per step; float64 product + sum then one rounding models it
        q = (q.astype(np.float64) * t + np.float64(ci)).astype(np.float32)
    err = np.abs(q.astype(np.float64) - np.cos(x.astype(np.float64))).max()
    assert err <= 4.5e-7, err
