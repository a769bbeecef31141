"""CPU checks of the oracle restatements that the GPU parity tests lean on:
each against a direct definition on tiny inputs, or an exact property."""
import numpy as np

from oracle import lightfield as olf
from oracle import propagation as oprop
from oracle import reconstruct as orec
from oracle import wrp as owrp


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _field(ny, nx, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))


def test_fresnel_conv_equals_direct_linear_convolution():
    """2x zero-padded FFT convolution == the linear convolution with the
    sampled impulse response h(x, y) = e^{ikz}/(i lambda z) e^{i pi (x^2+y^2)/(lambda z)} dp^2."""
    ny, nx, dp, lam, z = 6, 5, 8e-6, 532e-9, 0.003
    U = _field(ny, nx, 1)
    k = 2 * np.pi / lam
    out = np.zeros((ny, nx), np.complex128)
    for r in range(ny):
        for c in range(nx):
            for r2 in range(ny):
                for c2 in range(nx):
                    x, y = (c - c2) * dp, (r - r2) * dp
                    h = np.exp(1j * k * z) / (1j * lam * z) * np.exp(1j * np.pi * (x * x + y * y) / (lam * z)) * dp * dp
                    out[r, c] += U[r2, c2] * h
    assert rel(owrp.fresnel_conv(U, dp, lam, z), out) < 1e-12


def test_fresnel_tf_round_trip():
    """The transfer function is unimodular: +z then -z gives the input back."""
    U = _field(8, 12, 2)
    V = owrp.fresnel_tf(owrp.fresnel_tf(U, 8e-6, 6e-6, 0.01, 532e-9), 8e-6, 6e-6, -0.01, 532e-9)
    assert rel(V, U) < 1e-12


def test_as_bandlimited_identity_at_zero_distance():
    for shape in [(8, 8), (7, 9)]:
        U = _field(*shape, 3)
        assert rel(oprop.as_bandlimited(U, 8e-6, 8e-6, 0.0, 532e-9), U) < 1e-12


def test_lightfield_centre_convention():
    """A flat view with zero phase transforms to nu nv at the centre sample
    (nv // 2, nu // 2) of its block and zero elsewhere."""
    nt, ns, nv, nu = 2, 3, 5, 4
    lf = np.zeros((nt, ns, nv, nu))
    lf[1, 2] = 1.0
    out = olf.lightfield_to_field(lf, np.zeros_like(lf))
    expect = np.zeros((nt * nv, ns * nu), np.complex128)
    expect[1 * nv + nv // 2, 2 * nu + nu // 2] = nv * nu
    assert np.allclose(out, expect, atol=1e-12)


def test_eye_shift_is_the_reference_rotation():
    """The reference's CPU fftShift moves in[i] to out[(i - n/2) mod n]."""
    for n in (6, 7):
        a = np.arange(n * (n + 1)).reshape(n + 1, n).astype(float)
        s = orec._s(a)
        for i in range(n + 1):
            for j in range(n):
                assert s[(i - (n + 1) // 2) % (n + 1), (j - n // 2) % n] == a[i, j]


def test_wrp_window_single_point():
    """One point on the axis: an N x N window of e^{i ph} e^{ikr}/r, N odd
    from the MATLAB size rule, its zero offset at 0-based index cx - 1."""
    lam, dp, res, z_wrp, ph = 532e-9, 8e-6, 31, 0.0, 0.7
    obj = np.array([[0.0, 0.0, -0.002]])
    holo = owrp.fn_wrp_window(obj, lam, dp, res, z_wrp, phase=np.array([ph]))
    dz = z_wrp - obj[0, 2]
    n = int(np.floor(abs(lam * dz / dp ** 2 / 2) + 0.5 + 0.5) * 2 - 1)
    c = (res - 1) // 2 - 1
    k = 2 * np.pi / lam
    assert abs(holo[c, c] - np.exp(1j * ph) * np.exp(1j * k * dz) / dz) < 1e-9 * abs(holo[c, c])
    r = np.sqrt(dz * dz + dp * dp)
    assert abs(holo[c + 1, c] - np.exp(1j * ph) * np.exp(1j * k * r) / r) < 1e-9 * abs(holo[c, c])
    nz = np.flatnonzero(np.abs(holo).sum(axis=1))
    assert len(nz) == min(n, res) and n % 2 == 1
