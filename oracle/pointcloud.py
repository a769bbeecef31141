"""ctypes access to the C oracle (pointcloud.c) and, when built, to the
reference's own point-cloud library in _ref/ — TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _b


class KetiSpec(C.Structure):
    _fields_ = [("scale_x", C.c_float), ("scale_y", C.c_float), ("scale_z", C.c_float), ("offset_depth", C.c_float),
                ("pitch_x", C.c_float), ("pitch_y", C.c_float), ("nx", C.c_int), ("ny", C.c_int),
                ("lambda_", C.c_float), ("tilt_x", C.c_float), ("tilt_y", C.c_float)]


class PcParams(C.Structure):
    _fields_ = [("scale_x", C.c_double), ("scale_y", C.c_double), ("scale_z", C.c_double),
                ("offset_depth", C.c_double), ("pitch_x", C.c_double), ("pitch_y", C.c_double),
                ("nx", C.c_int), ("ny", C.c_int), ("lambda_", C.c_double), ("tilt_x_deg", C.c_double),
                ("tilt_y_deg", C.c_double)]


_or = None


def lib():
    global _or
    if _or is None:
        _or = C.CDLL(str(_b.build_oracle()))
        _or.oracle_keti_f32.argtypes = [C.c_void_p, C.c_int, C.POINTER(KetiSpec), C.c_void_p]
        _or.oracle_pc_f64.argtypes = [C.c_void_p, C.c_int, C.POINTER(PcParams), C.c_void_p, C.c_int, C.c_int]
        _or.oracle_fresnel_f64.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p]
        _or.oracle_wrp_f64.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                       C.c_int, C.c_void_p]
    return _or


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def keti_f32(xyza: np.ndarray, spec: dict, dst: np.ndarray | None = None) -> np.ndarray:
    """ophGenCghPointCloud restatement; dst accumulated (zeros if None)."""
    xyza = np.ascontiguousarray(xyza, dtype=np.float32)
    s = KetiSpec(spec["scale_x"], spec["scale_y"], spec["scale_z"], spec["offset_depth"], spec["pitch_x"],
                 spec["pitch_y"], spec["nx"], spec["ny"], spec["lambda"], spec["tilt_x"], spec["tilt_y"])
    if dst is None:
        dst = np.zeros((spec["ny"], spec["nx"]), dtype=np.float32)
    lib().oracle_keti_f32(_ptr(xyza), xyza.shape[0], C.byref(s), _ptr(dst))
    return dst


def pc_f64(xyza: np.ndarray, spec: dict, row0: int = 0, nrows: int | None = None) -> np.ndarray:
    """Exact-r complex field in double; rows [row0, row0+nrows) evaluated."""
    xyza = np.ascontiguousarray(xyza, dtype=np.float64)
    p = PcParams(spec["scale_x"], spec["scale_y"], spec["scale_z"], spec["offset_depth"], spec["pitch_x"],
                 spec["pitch_y"], spec["nx"], spec["ny"], spec["lambda"], spec["tilt_x"], spec["tilt_y"])
    nrows = spec["ny"] - row0 if nrows is None else nrows
    out = np.zeros((spec["ny"], spec["nx"], 2), dtype=np.float64)
    lib().oracle_pc_f64(_ptr(xyza), xyza.shape[0], C.byref(p), _ptr(out), row0, nrows)
    return out[..., 0] + 1j * out[..., 1]


def fresnel_f64(xyza, nx, ny, dp, lam) -> np.ndarray:
    xyza = np.ascontiguousarray(xyza, dtype=np.float64)
    out = np.zeros((ny, nx, 2), dtype=np.float64)
    lib().oracle_fresnel_f64(_ptr(xyza), xyza.shape[0], nx, ny, dp, lam, _ptr(out))
    return out[..., 0] + 1j * out[..., 1]


def wrp_f64(xyz, nx, ny, dp, lam, z, fixed_w=0) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    out = np.zeros((ny, nx, 2), dtype=np.float64)
    lib().oracle_wrp_f64(_ptr(xyz), xyz.shape[0], nx, ny, dp, lam, z, fixed_w, _ptr(out))
    return out[..., 0] + 1j * out[..., 1]


# ---- the reference itself (built only where its sources exist) ----------

_ref = None


def reference_available() -> bool:
    try:
        return _reference() is not None
    except Exception:
        return False


def _reference(omp: bool = False):
    global _ref
    path = (_b.REF_OUT / ("libketi_ref_omp.so" if omp else "libketi_ref.so"))
    if not path.exists():
        if _b.build_reference() is None:
            return None
    L = C.CDLL(str(path))
    L.keti_ref_gen.restype = C.c_double
    L.keti_ref_gen.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.keti_ref_load_points.argtypes = [C.c_char_p, C.c_void_p, C.c_int]
    L.keti_ref_load_spec.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p]
    return L


def reference_keti(xyza: np.ndarray, spec: dict, omp: bool = False) -> np.ndarray:
    L = _reference(omp)
    if L is None:
        raise RuntimeError("reference point-cloud library not built (reference sources absent)")
    xyza = np.ascontiguousarray(xyza, dtype=np.float32)
    s11 = np.array([spec["scale_x"], spec["scale_y"], spec["scale_z"], spec["offset_depth"], spec["pitch_x"],
                    spec["pitch_y"], spec["lambda"], spec["tilt_x"], spec["tilt_y"], 0, 0], dtype=np.float32)
    dst = np.zeros((spec["ny"], spec["nx"]), dtype=np.float32)
    L.keti_ref_gen(_ptr(xyza), xyza.shape[0], _ptr(s11), spec["nx"], spec["ny"], _ptr(dst))
    return dst
