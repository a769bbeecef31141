"""The point-light-source oracle against its own identities (no GPU).

cwoPLS cannot be built here (it needs the CWO base class and the absent
CWO++ DLL), so these checks pin the restatement by properties instead of
reference outputs: the separable form equals the per-term Fresnel sum,
CGHFresnel is its real part, and Huygens approaches the paraxial sum times
e^{ikz}/z far from the points.
"""
import numpy as np

from openholo_gb300 import scenes
from oracle import pls as opls


def _geom():
    return dict(nx=40, ny=33, dpx=8e-6, dpy=6e-6, lam=532e-9)


def test_separable_equals_term_sum():
    pts = scenes.pls_scene(1, 60, xy_half=0.1e-3, z_range=(0.02, 0.03))
    g = _geom()
    for use_amp in (False, True):
        a = opls.pls(pts, mode=opls.FRESNEL, z=0.01, ph=0.3, dox=1e-5, doy=-2e-5, sox=3e-6, soy=0.0,
                     use_amplitude=use_amp, **g)
        b = opls.pls_fresnel_separable(pts, z=0.01, ph=0.3, dox=1e-5, doy=-2e-5, sox=3e-6, soy=0.0,
                                       use_amplitude=use_amp, **g)
        assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max()


def test_cgh_fresnel_is_real_part():
    pts = scenes.pls_scene(2, 50, xy_half=0.1e-3, z_range=(0.02, 0.03))
    g = _geom()
    u = opls.pls(pts, mode=opls.FRESNEL, z=0.0, ph=1.1, **g)
    i = opls.pls(pts, mode=opls.CGH_FRESNEL, z=0.0, ph=1.1, **g)
    assert i.dtype == np.float64 and np.allclose(i, u.real, rtol=0, atol=1e-12)


def test_huygens_paraxial_limit():
    # one point on axis far away: exp(ikr)/r -> exp(ikz)/z exp(ik rho^2/(2z))
    pts = np.array([[1.0, 0.0, 0.0, 0.0, 0.5]], np.float32)
    g = _geom()
    lam = g["lam"]
    h = opls.pls(pts, mode=opls.HUYGENS, z=0.0, **g)
    f = opls.pls(pts, mode=opls.FRESNEL, z=0.0, **g)
    k = 2 * np.pi / lam
    ratio = h * 0.5 / np.exp(1j * k * 0.5) / f
    assert np.abs(ratio - 1).max() < 1e-3


def test_texdep_single_equals_convolution():
    """cwoTexDep::WRP(z) oracle: the per-texel scatter equals the 2-D
    convolution of the texture with the separable zone-plate window (the
    identity the GPU kernel is built on)."""
    from scipy.signal import convolve2d
    from oracle import texdep as otd
    rng = np.random.default_rng(4)
    tex = (rng.random((20, 26)) * 256).astype(np.uint8)
    z, px, py, lam = 1.2e-3, 8e-6, 6e-6, 532e-9
    w = otd.half_width(z, lam, px)
    k = 2 * np.pi / float(np.float32(lam))
    off = np.arange(-w, w)
    kern = np.exp(1j * k * (z + ((off[None, :] * float(np.float32(px))) ** 2 +
                                 (off[:, None] * float(np.float32(py))) ** 2) / (2 * z)))
    full = convolve2d(tex.astype(np.complex128), kern)     # output index = texel + (off + w)
    conv = full[w:w + 20, w:w + 26]
    ref = otd.wrp_single(tex, px, py, lam, z)
    assert np.abs(conv - ref).max() < 1e-9 * np.abs(ref).max()
