"""Encoders, uint8 normalisation, WRP accumulation and Fresnel propagation on
the GPU against CPU restatements (oracle)."""
import ctypes as C
import math

import numpy as np
import pytest
import torch

from openholo_gb300 import _lib, scenes
from openholo_gb300._lib import WrpParams
from oracle import depthmap as odm
from oracle import encoding as oenc
from oracle import pointcloud as opc
from oracle import propagation as oprop
from oracle import wrp as owrp

pytestmark = pytest.mark.gpu


def S():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def field_sample(ny=48, nx=64, seed=0):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))


KINDS = {0: "real", 1: "p2a", 2: "ni", 3: "burckhardt", 4: "two_phase", 5: "ssb_left", 6: "ssb_right",
         7: "ssb_top", 8: "ssb_bottom", 9: "phase_only_u8", 10: "amplitude"}


@pytest.mark.parametrize("kind", sorted(KINDS))
def test_encoders(ctx, kind):
    U = field_sample()
    ny, nx = U.shape
    t = torch.from_numpy(U).cuda()
    width = {3: 3, 4: 2}.get(kind, 1)
    out = torch.empty((ny, nx * width), dtype=torch.uint8 if kind == 9 else torch.float64, device="cuda")
    _lib.call("oh_encode", ctx.handle, 1, kind, nx, ny, C.c_void_p(t.data_ptr()), C.c_void_p(out.data_ptr()), S())
    torch.cuda.synchronize()
    ref = oenc.encode(U, KINDS[kind])
    got = out.cpu().numpy()
    if kind == 9:
        assert np.abs(got.astype(int) - ref.astype(int)).max() <= 1
        assert np.mean(got != ref) < 1e-3
    else:
        assert np.allclose(got, ref, rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("round_half", [0, 1])
def test_normalize_u8(ctx, round_half):
    f = np.random.default_rng(2).standard_normal((40, 50))
    t = torch.from_numpy(f).cuda()
    out = torch.empty((40, 50), dtype=torch.uint8, device="cuda")
    _lib.call("oh_normalize_u8", ctx.handle, 1, 50, 40, C.c_void_p(t.data_ptr()), C.c_void_p(out.data_ptr()),
              round_half, S())
    torch.cuda.synchronize()
    ref = oenc.keti_normalize(f.astype(np.float32)) if round_half else odm.normalize_u8(f)
    assert np.array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("fixed_w,precision,plane,gap", [(8, "fp64", (96, 80), 0.4e-3), (8, "fp32", (96, 80), 0.4e-3),
                                                        (0, "fp64", (96, 80), 0.4e-3),
                                                        (40, "fp32", (300, 170), 0.4e-3),
                                                        (40, "fp64", (300, 170), 0.4e-3),
                                                        (3, "fp32", (257, 129), 0.4e-3),
                                                        (24, "fp32", (300, 170), 5e-3),
                                                        (24, "fp32", (300, 170), -5e-3)])
def test_wrp_accumulate(ctx, fixed_w, precision, plane, gap):
    # windows straddle 64x64 tiles and the plane's edges; some centres lie outside the plane.
    # gap 5 mm (either side of the points) makes the FP32 windows paraxial enough for the series form.
    nx, ny = plane
    pts = scenes.wrp_scene(4, 200 if nx < 100 else 1500, box=(nx * 9e-6, ny * 9e-6, 0.2e-3), zc=0.01)
    dp, lam = 8e-6, 532e-9
    if gap > 0:
        z = 0.01 - 0.1e-3 - gap if fixed_w else 0.012   # dz < 0; formula mode: dz ~ 2 mm -> w ~ 15
    else:
        z = 0.01 + 0.1e-3 - gap                         # plane on the other side of the points (dz > 0)
    p = WrpParams(nx, ny, dp, lam, z, fixed_w)
    tp = torch.from_numpy(pts).cuda()
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    w = torch.zeros((ny, nx), dtype=cdt, device="cuda")
    _lib.call("oh_wrp_accumulate", ctx.handle, 1 if precision == "fp64" else 0, C.byref(p),
              C.c_void_p(tp.data_ptr()), pts.shape[0], C.c_void_p(w.data_ptr()), S())
    torch.cuda.synchronize()
    ref = opc.wrp_f64(pts, nx, ny, dp, lam, z, fixed_w)
    tol = 1e-9 if precision == "fp64" else 1e-4
    assert np.linalg.norm(w.cpu().numpy() - ref) <= tol * np.linalg.norm(ref)


def _wrp_run(ctx, pts, nx, ny, dp, lam, z, w, engine=None, kernels=None):
    """One oh_wrp_accumulate call; `kernels` (a set) receives the names of the
    library's timed kernels that ran."""
    import os
    p = WrpParams(nx, ny, dp, lam, z, w)
    tp = torch.from_numpy(pts).cuda()
    out = torch.zeros((ny, nx), dtype=torch.complex64, device="cuda")
    old = os.environ.get("OH_WRP_ENGINE")
    if engine:
        os.environ["OH_WRP_ENGINE"] = engine
    try:
        ctx.set_timing(True)
        ctx.read_timing(reset=True)
        _lib.call("oh_wrp_accumulate", ctx.handle, 0, C.byref(p), C.c_void_p(tp.data_ptr()), pts.shape[0],
                  C.c_void_p(out.data_ptr()), S())
        torch.cuda.synchronize()
        if kernels is not None:
            kernels.update(ctx.read_timing(reset=True).keys())
    finally:
        ctx.set_timing(False)
        if engine:
            if old is None:
                del os.environ["OH_WRP_ENGINE"]
            else:
                os.environ["OH_WRP_ENGINE"] = old
    from openholo_gb300._lib import lib
    assert lib().oh_ctx_device_status(ctx.handle, S()) == 0
    return out.cpu().numpy()


@pytest.mark.parametrize("plane,npts,w,gap", [((300, 170), 1500, 24, 5e-3), ((257, 200), 900, 32, -6e-3),
                                             ((64, 300), 400, 16, 8e-3)])
def test_wrp_tensor_form(ctx, plane, npts, w, gap):
    """Fixed windows far enough from the points to be separable run as the
    tcgen05 GEMM (BF16 hi/lo, rank-2 separable terms): against the FP64
    oracle and against the direct FP32 tile kernel.  Windows straddle the
    128 x 64 regions and the plane's edges; some centres lie outside."""
    nx, ny = plane
    dp, lam = 3.74e-6, 532e-9
    pts = scenes.wrp_scene(8, npts, box=(nx * 4.2e-6, ny * 4.2e-6, 1e-3), zc=0.01)
    z = 0.01 - 0.5e-3 - gap if gap > 0 else 0.01 + 0.5e-3 - gap
    ran, ran_direct = set(), set()
    tc = _wrp_run(ctx, pts, nx, ny, dp, lam, z, w, kernels=ran)
    direct = _wrp_run(ctx, pts, nx, ny, dp, lam, z, w, engine="direct", kernels=ran_direct)
    assert "wrp_tc" in ran and "wrp_tc" not in ran_direct
    ref = opc.wrp_f64(pts, nx, ny, dp, lam, z, w)
    assert np.linalg.norm(tc - ref) <= 5e-5 * np.linalg.norm(ref)
    assert np.linalg.norm(tc - direct) <= 5e-5 * np.linalg.norm(ref)


def test_wrp_tensor_and_direct_points_mixed(ctx):
    """Points near the plane (not separable: direct kernel) and far from it
    (tensor form) in one call: both parts land in the same plane."""
    nx, ny, dp, lam, w = 200, 180, 3.74e-6, 532e-9, 24
    far = scenes.wrp_scene(9, 700, box=(nx * 4.2e-6, ny * 4.2e-6, 1e-3), zc=0.01)
    near = scenes.wrp_scene(10, 300, box=(nx * 4.2e-6, ny * 4.2e-6, 0.2e-3), zc=0.0146)
    pts = np.concatenate([far, near])
    z = 0.015
    ran = set()
    got = _wrp_run(ctx, pts, nx, ny, dp, lam, z, w, kernels=ran)
    assert "wrp_tc" in ran
    ref = opc.wrp_f64(pts, nx, ny, dp, lam, z, w)
    assert np.linalg.norm(got - ref) <= 5e-5 * np.linalg.norm(ref)


def test_wrp_tensor_form_full_size(ctx):
    """The 200,000-point, 3840 x 2160, 64 x 64 window workload: the tensor
    form against the direct kernel (the oracle is too slow at this size)."""
    nx, ny, dp, lam, w = 3840, 2160, 3.74e-6, 532e-9, 32
    pts = scenes.wrp_scene(12, 200_000)
    z = float(pts[:, 2].min()) - 5e-3
    ran = set()
    tc = _wrp_run(ctx, pts, nx, ny, dp, lam, z, w, kernels=ran)
    direct = _wrp_run(ctx, pts, nx, ny, dp, lam, z, w, engine="direct")
    assert "wrp_tc" in ran
    assert np.linalg.norm(tc - direct) <= 5e-5 * np.linalg.norm(direct)


@pytest.mark.parametrize("shape", [(64, 64), (48, 80)])
def test_fresnel_propagate(ctx, shape):
    ny, nx = shape
    U = field_sample(ny, nx, 7)
    dp, lam, z = 8e-6, 532e-9, 0.02
    for precision, tol in (("fp64", 1e-10), ("fp32", 1e-4)):
        t = torch.from_numpy(U).to(torch.complex128 if precision == "fp64" else torch.complex64).cuda()
        _lib.call("oh_fresnel_propagate", ctx.handle, 1 if precision == "fp64" else 0, nx, ny, dp, lam, z,
                  C.c_void_p(t.data_ptr()), S())
        torch.cuda.synchronize()
        ref = owrp.fresnel_conv(U, dp, lam, z)
        assert np.linalg.norm(t.cpu().numpy() - ref) <= tol * np.linalg.norm(ref), precision


@pytest.mark.parametrize("shape", [(540, 960), (512, 512), (1080, 960), (540, 1920), (512, 1024), (512, 2048),
                                   (1080, 2160)])
def test_fresnel_propagate_separable(ctx, shape):
    """FP32 sizes whose padded lengths have compile-time FFT schedules run the
    three-pass separable path; it must equal the padded-grid oracle, and
    alternating distances must rebuild its cached tables."""
    ny, nx = shape
    U = field_sample(ny, nx, 9)
    dp, lam = 3.74e-6, 532e-9
    for z in (5e-3, 7e-3, 5e-3):
        t = torch.from_numpy(U).to(torch.complex64).cuda()
        _lib.call("oh_fresnel_propagate", ctx.handle, 0, nx, ny, dp, lam, z, C.c_void_p(t.data_ptr()), S())
        torch.cuda.synchronize()
        ref = owrp.fresnel_conv(U, dp, lam, z)
        err = np.linalg.norm(t.cpu().numpy() - ref) / np.linalg.norm(ref)
        assert err <= 1e-5, (z, err)


def test_fresnel_propagate_separable_3840x2160(ctx):
    """The separable path at the WRP hologram size (padded lengths 7680 and
    4320: radix-30 and radix-18 stages) against the padded-grid oracle."""
    ny, nx = 2160, 3840
    U = field_sample(ny, nx, 11)
    dp, lam, z = 3.74e-6, 532e-9, 6e-3
    t = torch.from_numpy(U).to(torch.complex64).cuda()
    _lib.call("oh_fresnel_propagate", ctx.handle, 0, nx, ny, dp, lam, z, C.c_void_p(t.data_ptr()), S())
    torch.cuda.synchronize()
    ref = owrp.fresnel_conv(U, dp, lam, z)
    err = np.linalg.norm(t.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert err <= 1e-5, err


def test_fresnel_point_focus(ctx):
    """Known answer: a WRP point field propagated back by -z refocuses to a spot."""
    n, dp, lam, z = 128, 8e-6, 532e-9, 0.03
    U = np.zeros((n, n), np.complex128)
    U[n // 2, n // 2] = 1.0
    t = torch.from_numpy(U).cuda()
    _lib.call("oh_fresnel_propagate", ctx.handle, 1, n, n, dp, lam, z, C.c_void_p(t.data_ptr()), S())
    _lib.call("oh_fresnel_propagate", ctx.handle, 1, n, n, dp, lam, -z, C.c_void_p(t.data_ptr()), S())
    torch.cuda.synchronize()
    back = np.abs(t.cpu().numpy())
    assert np.unravel_index(np.argmax(back), back.shape) == (n // 2, n // 2)


def test_fresnel_spectrum_cache_follows_distance(ctx):
    """Alternating propagation distances reuse one cached spectrum slot
    correctly (results equal the oracle for each distance)."""
    ny, nx = 48, 64
    U = field_sample(ny, nx, 3)
    dp, lam = 8e-6, 532e-9
    for z in (0.02, 0.035, 0.02):
        t = torch.from_numpy(U).cuda()
        _lib.call("oh_fresnel_propagate", ctx.handle, 1, nx, ny, dp, lam, z, C.c_void_p(t.data_ptr()), S())
        torch.cuda.synchronize()
        ref = owrp.fresnel_conv(U, dp, lam, z)
        assert np.linalg.norm(t.cpu().numpy() - ref) <= 1e-10 * np.linalg.norm(ref), z


@pytest.mark.parametrize("shape,dx,dy,z,lam", [((48, 64), 8e-6, 8e-6, 0.05, 532e-9),       # band limit active
                                               ((33, 45), 6e-6, 9e-6, -0.02, 633e-9),      # odd sizes, z < 0
                                               ((40, 40), 0.2e-6, 0.2e-6, 2e-6, 532e-9)])  # evanescent region
def test_propagate_as_bandlimited(ctx, shape, dx, dy, z, lam):
    ny, nx = shape
    U = field_sample(ny, nx, 11)
    ref = oprop.as_bandlimited(U, dx, dy, z, lam)
    for precision, tol in (("fp64", 1e-10), ("fp32", 1e-5)):
        t = torch.from_numpy(U).to(torch.complex128 if precision == "fp64" else torch.complex64).cuda()
        _lib.call("oh_propagate", ctx.handle, 1 if precision == "fp64" else 0, _lib.PROP_AS_BANDLIMITED, nx, ny,
                  dx, dy, z, lam, C.c_void_p(t.data_ptr()), S())
        torch.cuda.synchronize()
        got = t.cpu().numpy()
        assert np.linalg.norm(got - ref) <= tol * np.linalg.norm(ref), precision


@pytest.mark.parametrize("shape,z", [((48, 64), 0.05), ((33, 45), -0.03), ((540, 960), 0.05)])
def test_propagate_fresnel_tf(ctx, shape, z):
    ny, nx = shape
    U = field_sample(ny, nx, 12)
    dx, dy, lam = 8e-6, 6e-6, 532e-9
    ref = owrp.fresnel_tf(U, dx, dy, z, lam)
    for precision, tol in (("fp64", 1e-10), ("fp32", 1e-5)):
        t = torch.from_numpy(U).to(torch.complex128 if precision == "fp64" else torch.complex64).cuda()
        _lib.call("oh_propagate", ctx.handle, 1 if precision == "fp64" else 0, _lib.PROP_FRESNEL_TF, nx, ny,
                  dx, dy, z, lam, C.c_void_p(t.data_ptr()), S())
        torch.cuda.synchronize()
        assert np.linalg.norm(t.cpu().numpy() - ref) <= tol * np.linalg.norm(ref), precision


@pytest.mark.parametrize("res,precision", [(65, "fp64"), (65, "fp32"), (64, "fp32")])
def test_wrp_matlab_window(ctx, res, precision):
    """fn_wrp.m: odd centred windows, random phase given per point, 1/r; some
    windows run off the plane."""
    dp, lam, z_wrp = 10e-6, 532e-9, 5e-3
    u = scenes.uniform(21, 3, 40 * 4).reshape(40, 4)
    obj = np.empty((40, 3))
    obj[:, 0] = (u[:, 0] - 0.5) * res * dp * 1.2
    obj[:, 1] = (u[:, 1] - 0.5) * res * dp * 1.2
    obj[:, 2] = 1e-3 + u[:, 2] * 2e-3
    phase = u[:, 3] * 2 * np.pi
    ref = owrp.fn_wrp_window(obj, lam, dp, res, z_wrp, phase)
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    holo = torch.zeros((res, res), dtype=cdt, device="cuda")
    t_obj = torch.from_numpy(obj).cuda()
    t_ph = torch.from_numpy(phase).cuda()
    _lib.call("oh_wrp_matlab", ctx.handle, 1 if precision == "fp64" else 0, res, dp, lam, z_wrp,
              C.c_void_p(t_obj.data_ptr()), C.c_void_p(t_ph.data_ptr()), 40, C.c_void_p(holo.data_ptr()), S())
    torch.cuda.synchronize()
    tol = 1e-10 if precision == "fp64" else 1e-5
    assert np.linalg.norm(holo.cpu().numpy() - ref) <= tol * np.linalg.norm(ref)


@pytest.mark.parametrize("method", [_lib.PROP_FRESNEL_TF, _lib.PROP_AS_BANDLIMITED])
@pytest.mark.parametrize("z", [1e-3, 5e-3])
def test_propagation_round_trip(ctx, method, z):
    # known answer: propagating a compact beam by +z and then by -z returns it
    # (the transfer function is unitary; the band-limited form loses nothing
    # for a beam that stays inside the window at these distances)
    ny, nx = 64, 96
    y, x = np.mgrid[0:ny, 0:nx]
    g = np.exp(-(((x - nx / 2) / 6.0) ** 2 + ((y - ny / 2) / 5.0) ** 2)) * np.exp(1j * 0.3 * x)
    for precision, tol in (("fp64", 1e-9), ("fp32", 1e-5)):
        t = torch.from_numpy(g).to(torch.complex128 if precision == "fp64" else torch.complex64).cuda()
        for zz in (z, -z):
            _lib.call("oh_propagate", ctx.handle, 1 if precision == "fp64" else 0, method, nx, ny, 8e-6, 8e-6, zz,
                      532e-9, C.c_void_p(t.data_ptr()), S())
        torch.cuda.synchronize()
        back = t.cpu().numpy().astype(np.complex128)
        assert np.linalg.norm(back - g) <= tol * np.linalg.norm(g), precision
