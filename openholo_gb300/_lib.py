"""ctypes binding of the C ABI declared in include/oh.h.

Loading fails loudly when liboh_gb300.so has not been built: there is no
fallback implementation behind this module.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "liboh_gb300.so"

OH_OK = 0
OH_FP32, OH_FP64 = 0, 1
OH_PHASE_REFERENCE, OH_PHASE_ARRAY, OH_PHASE_SEEDED = 0, 1, 2

STATUS = {0: "OH_OK", 1: "OH_ERR_INVALID_ARG", 2: "OH_ERR_UNSUPPORTED_SIZE", 3: "OH_ERR_CUDA",
          4: "OH_ERR_ALLOC", 5: "OH_ERR_TIMEOUT", 6: "OH_ERR_IO"}


class OhError(RuntimeError):
    def __init__(self, status: int, func: str, msg: str):
        super().__init__(f"{func} -> {STATUS.get(status, status)}: {msg}")
        self.status = status


class DepthmapParams(C.Structure):
    """oh_depthmap_params (include/oh.h)."""
    _fields_ = [
        ("pnx", C.c_int), ("pny", C.c_int),
        ("ppx", C.c_double), ("ppy", C.c_double),
        ("lambda_", C.c_double), ("field_lens", C.c_double),
        ("near_depthmap", C.c_double), ("far_depthmap", C.c_double),
        ("num_of_depth", C.c_int), ("flag_change_depth_quantization", C.c_int),
        ("default_depth_quantization", C.c_int), ("transform_viewing_window", C.c_int),
        ("pad", C.c_int), ("sig_location_x", C.c_int), ("sig_location_y", C.c_int),
        ("phase_mode", C.c_int), ("seed", C.c_uint64),
        ("rand_phase_re", C.c_double), ("rand_phase_im", C.c_double),
        ("render_depth", C.POINTER(C.c_int)), ("n_render_depth", C.c_int),
    ]


class DepthmapFrame(C.Structure):
    """oh_depthmap_frame (include/oh.h)."""
    _fields_ = [("params", DepthmapParams), ("img", C.c_void_p), ("depth", C.c_void_p), ("phase", C.c_void_p),
                ("fringe", C.c_void_p), ("field", C.c_void_p)]


BATCH_GRAPH = 1
PROP_FRESNEL_TF, PROP_AS_BANDLIMITED = 0, 1


class PcParams(C.Structure):
    """oh_pc_params (include/oh.h), field order of OphSpec."""
    _fields_ = [
        ("scale_x", C.c_double), ("scale_y", C.c_double), ("scale_z", C.c_double),
        ("offset_depth", C.c_double), ("pitch_x", C.c_double), ("pitch_y", C.c_double),
        ("nx", C.c_int), ("ny", C.c_int), ("lambda_", C.c_double),
        ("tilt_x_deg", C.c_double), ("tilt_y_deg", C.c_double),
    ]


class WrpParams(C.Structure):
    """oh_wrp_params (include/oh.h)."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("pitch", C.c_double), ("lambda_", C.c_double),
                ("z_wrp", C.c_double), ("window", C.c_int)]


_vp = C.c_void_p
_i = C.c_int
_d = C.c_double

# name -> (restype, argtypes); every symbol declared in include/oh.h
class PlsParams(C.Structure):
    """oh_pls_params (include/oh.h)."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("dst_px", C.c_double), ("dst_py", C.c_double),
                ("dst_ox", C.c_double), ("dst_oy", C.c_double), ("src_ox", C.c_double), ("src_oy", C.c_double),
                ("lambda_", C.c_double), ("z", C.c_double), ("phase", C.c_double), ("mode", C.c_int),
                ("use_amplitude", C.c_int), ("engine", C.c_int)]


PLS_HUYGENS, PLS_FRESNEL, PLS_CGH_FRESNEL = 0, 1, 2
PLS_ENGINE_AUTO, PLS_ENGINE_DIRECT, PLS_ENGINE_GEMM, PLS_ENGINE_TENSOR = 0, 1, 2, 3


class UnetConfig(C.Structure):
    """oh_unet_config (include/oh.h)."""
    _fields_ = [("max_batch", C.c_int), ("max_height", C.c_int), ("max_width", C.c_int), ("seed", C.c_uint64),
                ("out_scale", C.c_float), ("depth_lut", C.c_float * 256)]


class SurrogateParams(C.Structure):
    """oh_surrogate_params (include/oh.h)."""
    _fields_ = [("dm", DepthmapParams), ("z_mid", C.c_double), ("psnr_threshold_db", C.c_float), ("check", C.c_int)]


class SurrogateReport(C.Structure):
    """oh_surrogate_report (include/oh.h)."""
    _fields_ = [("checked", C.c_int), ("fell_back", C.c_int), ("psnr_db", C.c_float), ("rel_err", C.c_float),
                ("max_abs_err", C.c_float), ("rms_err", C.c_float)]


class TexdepParams(C.Structure):
    """oh_texdep_params (include/oh.h)."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("px", C.c_double), ("py", C.c_double), ("lambda_", C.c_double),
                ("z", C.c_double), ("dz_step", C.c_double), ("range_lo", C.c_int), ("range_hi", C.c_int),
                ("dep_from_texture", C.c_int)]


TEXDEP_SINGLE, TEXDEP_RANGE = 0, 1


class EyeParams(C.Structure):
    """oh_eye_params (include/oh.h)."""
    _fields_ = [("pnx", C.c_int), ("pny", C.c_int), ("ppx", C.c_double), ("ppy", C.c_double),
                ("lambda_", C.c_double), ("field_lens", C.c_double), ("pixel_scale", C.c_int),
                ("eye_length", C.c_double), ("eye_pupil_diameter", C.c_double), ("eye_center_x", C.c_double),
                ("eye_center_y", C.c_double), ("focus_distance", C.c_double)]


class MeshParams(C.Structure):
    """oh_mesh_params (include/oh.h)."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("dx", C.c_double), ("dy", C.c_double), ("lambda_", C.c_double),
                ("illu", C.c_double * 3), ("continuous", C.c_int)]


SIGNATURES = {
    "oh_ctx_create": (_i, [C.POINTER(_vp), _i]),
    "oh_ctx_destroy": (_i, [_vp]),
    "oh_ctx_scratch_bytes": (C.c_size_t, [_vp]),
    "oh_ctx_release_scratch": (_i, [_vp]),
    "oh_status_string": (C.c_char_p, [_i]),
    "oh_last_error": (C.c_char_p, []),
    "oh_kernel_launch_count": (C.c_uint64, []),
    "oh_version": (C.c_char_p, []),
    "oh_ctx_set_timing": (_i, [_vp, _i]),
    "oh_ctx_device_status": (_i, [_vp, _vp]),
    "oh_ctx_set_test_stall": (_i, [_vp, _i, C.c_longlong]),
    "oh_ctx_set_depthmap_layer_limit": (_i, [_vp, C.c_size_t]),
    "oh_ctx_set_depthmap_batch_mode": (_i, [_vp, _i]),
    "oh_depthmap_autotune_batch": (_i, [_vp, _vp, _i, _i, _vp]),
    "oh_depthmap_batch_tuning": (_i, [_vp, _i, C.POINTER(_i), C.POINTER(_d)]),
    "oh_ctx_set_autotune_file": (_i, [_vp, C.c_char_p]),
    "oh_measure_issue_peaks": (_i, [_i, C.POINTER(_d), C.POINTER(_d), C.POINTER(_d), C.POINTER(_d)]),
    "oh_conv2d_bf16": (_i, [_vp, _i, _i, _i, _i, _i, _i, _i, _vp, _i, _vp, _vp, _i, _vp, _i, _vp, _i, _vp]),
    "oh_conv2d_wgrad_bf16": (_i, [_vp, _i, _i, _i, _i, _i, _i, _vp, _i, _vp, _i, _vp, _vp]),
    "oh_unet_config_default": (None, [_vp]),
    "oh_depthmap_propagate_field": (_i, [_vp, _i, _vp, _vp, _d, _vp, _vp, _vp, _vp]),
    "oh_scene_rgbd": (_i, [_vp, C.c_uint64, _i, _i, _i, _vp, _vp]),
    "oh_surrogate_mid_field": (_i, [_vp, _vp, _d, _vp, _vp, _vp]),
    "oh_surrogate_generate": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "oh_unet_create": (_i, [_vp, _vp, C.POINTER(_vp)]),
    "oh_unet_destroy": (_i, [_vp]),
    "oh_unet_param_count": (C.c_size_t, [_vp]),
    "oh_unet_get_params": (_i, [_vp, _vp]),
    "oh_unet_set_params": (_i, [_vp, _vp]),
    "oh_unet_get_grads": (_i, [_vp, _vp]),
    "oh_unet_forward": (_i, [_vp, _vp, _i, _i, _i, _vp, _vp]),
    "oh_unet_compute_grads": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp, _vp]),
    "oh_unet_adam_step": (_i, [_vp, C.c_float, C.c_float, C.c_float, C.c_float, _vp]),
    "oh_unet_train_step": (_i, [_vp, _vp, _vp, _i, _i, _i, C.c_float, _vp, _vp]),
    "oh_ctx_read_timing": (_i, [_vp, _i, C.POINTER(C.c_char_p), C.POINTER(_d), C.POINTER(C.c_long), _i]),
    "oh_fft_supported": (_i, [_i, _i]),
    "oh_fft2d": (_i, [_vp, _i, _i, _i, _vp, _vp, _i, _i, _i, _vp]),
    "oh_fft1d_rows": (_i, [_vp, _i, _i, _i, _vp, _vp, _i, _i, _vp]),
    "oh_depthmap_params_default": (None, [C.POINTER(DepthmapParams)]),
    "oh_depthmap_read_config": (_i, [C.c_char_p, C.POINTER(DepthmapParams)]),
    "oh_depthmap_generate": (_i, [_vp, _i, C.POINTER(DepthmapParams), _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "oh_depthmap_generate_host": (_i, [_vp, _i, C.POINTER(DepthmapParams), _vp, _vp, _vp, _vp, _vp]),
    "oh_depthmap_levels": (_i, [C.POINTER(DepthmapParams), _vp, _vp]),
    "oh_pointcloud": (_i, [_vp, _i, C.POINTER(PcParams), _vp, _i, _vp, _vp, _vp]),
    "oh_pointcloud_host": (_i, [_vp, _i, C.POINTER(PcParams), _vp, _i, _vp, _vp, _vp]),
    "oh_pointcloud_noalloc": (_i, [C.POINTER(PcParams), _vp, _i, _vp, _vp, _vp]),
    "oh_wrp_accumulate": (_i, [_vp, _i, C.POINTER(WrpParams), _vp, _i, _vp, _vp]),
    "oh_fresnel_propagate": (_i, [_vp, _i, _i, _i, _d, _d, _d, _vp, _vp]),
    "oh_pls": (_i, [_vp, _i, C.POINTER(PlsParams), _vp, _i, _vp, _vp]),
    "oh_propagate": (_i, [_vp, _i, _i, _i, _i, _d, _d, _d, _d, _vp, _vp]),
    "oh_wrp_matlab": (_i, [_vp, _i, _i, _d, _d, _d, _vp, _vp, _i, _vp, _vp]),
    "oh_texdep_wrp": (_i, [_vp, _i, _i, C.POINTER(TexdepParams), _vp, _vp, _vp, _vp]),
    "oh_reconstruct_eye": (_i, [_vp, _i, C.POINTER(EyeParams), _vp, _vp, _vp]),
    "oh_lightfield_to_field": (_i, [_vp, _i, _i, _i, _i, _i, _vp, _vp, C.c_uint64, _vp, _vp]),
    "oh_mesh_hologram": (_i, [_vp, C.POINTER(MeshParams), _vp, _i, _vp, _vp, _vp]),
    "oh_depthmap_generate_batch": (_i, [_vp, _i, C.POINTER(DepthmapFrame), _i, C.c_uint, _vp]),
    "oh_encode": (_i, [_vp, _i, _i, _i, _i, _vp, _vp, _vp]),
    "oh_normalize_u8": (_i, [_vp, _i, _i, _i, _vp, _vp, _i, _vp]),
}

_lib = None


def lib() -> C.CDLL:
    """Load liboh_gb300.so once; raise if it is missing or incomplete."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                          " (there is no non-CUDA implementation)")
    L = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)   # AttributeError if a declared symbol is not exported
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status: int, func: str) -> None:
    if status != OH_OK:
        msg = lib().oh_last_error().decode(errors="replace")
        raise OhError(status, func, msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args), name)


class Context:
    """Owns one oh_ctx (FFT plans + scratch arena) on a CUDA device."""

    def __init__(self, device: int = 0):
        h = _vp()
        call("oh_ctx_create", C.byref(h), device)
        self.handle = h

    def close(self) -> None:
        if getattr(self, "handle", None) is not None and self.handle.value:
            lib().oh_ctx_destroy(self.handle)
            self.handle = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def scratch_bytes(self) -> int:
        return int(lib().oh_ctx_scratch_bytes(self.handle))

    def set_timing(self, on: bool) -> None:
        call("oh_ctx_set_timing", self.handle, 1 if on else 0)

    def read_timing(self, reset: bool = True) -> dict:
        """{kernel name: (total ms, launches)} since the last reset."""
        cap = 64
        names = (C.c_char_p * cap)()
        ms = (C.c_double * cap)()
        cnt = (C.c_long * cap)()
        n = lib().oh_ctx_read_timing(self.handle, 1 if reset else 0, names, ms, cnt, cap)
        return {names[i].decode(): (ms[i], cnt[i]) for i in range(min(n, cap))}


def launch_count() -> int:
    return int(lib().oh_kernel_launch_count())


def measure_issue_peaks(device: int = 0) -> dict:
    """Issue-rate microbenchmarks (oh_measure_issue_peaks): scalar and packed
    FP32 FMA warp instructions per second and sin.approx results per second
    on `device`."""
    a, b, c, m = _d(), _d(), _d(), _d()
    call("oh_measure_issue_peaks", device, C.byref(a), C.byref(b), C.byref(c), C.byref(m))
    return {"ffma_warp_inst_per_s": a.value, "ffma2_warp_inst_per_s": b.value, "mufu_per_s": c.value,
            "fp32_fma_flops_per_s": max(2 * 32 * a.value, 2 * 64 * b.value), "sm_mhz_implied": m.value}
