"""CPU checks of the depth-map oracle and of the library's host-side logic.

The reference's depth-map CPU path cannot be compiled here (Qt + FFTW), so the
vectorised oracle (oracle/depthmap.py) is cross-checked against a second,
loop-level restatement written directly from the reference's loops
(HologramGenerator_CPU.cpp:117-218, 231-270, 332-344) with a direct DFT in
place of FFTW.
"""
import cmath
import math

import numpy as np
import pytest

from oracle import depthmap as odm


def _fftshift_cpu(nx, ny, a):
    # HologramGenerator::fftShift (HologramGenerator_CPU.cpp:332-344)
    out = [[0j] * nx for _ in range(ny)]
    for i in range(nx):
        for j in range(ny):
            ti = i - nx // 2
            ti += nx if ti < 0 else 0
            tj = j - ny // 2
            tj += ny if tj < 0 else 0
            out[tj][ti] = a[j][i]
    return out


def _dft2(a, sign):
    ny, nx = len(a), len(a[0])
    out = [[0j] * nx for _ in range(ny)]
    for ky in range(ny):
        for kx in range(nx):
            s = 0j
            for y in range(ny):
                for x in range(nx):
                    s += a[y][x] * cmath.exp(sign * 2j * math.pi * (kx * x / nx + ky * y / ny))
            out[ky][kx] = s
    return out


def _loop_reference(img, depth, p: odm.DMParams, phase=None):
    """Literal loop restatement of Calc_Holo_CPU + encoding_CPU on a padded grid."""
    pny, pnx = img.shape
    P = p.pad
    Px, Py = P * pnx, P * pny
    ox, oy = (Px - pnx) // 2, (Py - pny) // 2
    lut = odm.depth_lut(p)
    zt = odm.transformed_levels(p)
    k = 2 * math.pi / p.lam
    ssx, ssy = Px * p.ppx, Py * p.ppy
    U = [[0j] * Px for _ in range(Py)]
    for dtr in range(1, p.num_of_depth + 1):
        u = [[0j] * Px for _ in range(Py)]
        tot = 0.0
        for r in range(pny):
            for c in range(pnx):
                a = img[r, c] / 255.0 * (1 if img[r, c] > 0 else 0) * (1.0 if lut[depth[r, c]] == dtr else 0.0)
                if phase is not None:
                    a = a * cmath.exp(1j * float(phase[r, c]))
                u[oy + r][ox + c] = a
                tot += abs(a)
        if tot == 0:
            continue
        z = zt[dtr - 1]
        carrier = complex(math.cos(k * z), math.sin(k * z))
        for r in range(Py):
            for c in range(Px):
                u[r][c] = u[r][c] * p.rand_phase * carrier
        S = _fftshift_cpu(Px, Py, _dft2(_fftshift_cpu(Px, Py, u), -1))
        for y in range(Py):
            for x in range(Px):
                fxx = (-1.0 / (2.0 * p.ppx)) + (1.0 / ssx) * x
                fyy = (1.0 / (2.0 * p.ppy)) - (1.0 / ssy) - (1.0 / ssy) * y
                sval = math.sqrt(1 - (p.lam * fxx) ** 2 - (p.lam * fyy) ** 2) * (k * -z)
                U[y][x] += cmath.exp(1j * sval) * S[y][x]
    cx1, cx2, cy1, cy2 = odm.crop_window(Px, Py, p.sig_location)
    crop = [[U[y][x] if (cx1 <= x <= cx2 and cy1 <= y <= cy2) else 0j for x in range(Px)] for y in range(Py)]
    h = _fftshift_cpu(Px, Py, _dft2(_fftshift_cpu(Px, Py, crop), +1))
    out = np.zeros((pny, pnx))
    for r in range(pny):
        for c in range(pnx):
            v = h[oy + r][ox + c] / (Px * Py)
            yy = (pny * p.ppy / 2.0) - p.ppy * r - p.ppy
            shift = cmath.exp(1j * 2 * math.pi * (yy / (4 * p.ppy))) if p.sig_location[1] == 1 else 1
            out[r, c] = (v * shift).real
    return out


def _tiny(seed, ny, nx):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, size=(ny, nx)).astype(np.uint8)
    img[rng.random((ny, nx)) < 0.2] = 0
    depth = rng.integers(0, 256, size=(ny, nx)).astype(np.uint8)
    return img, depth


@pytest.mark.parametrize("pad", [1, 2])
def test_oracle_matches_loop_restatement(pad):
    img, depth = _tiny(3, 6, 8)
    p = odm.DMParams(pnx=8, pny=6, num_of_depth=4, pad=pad, near=0.3, far=0.35)
    phase = np.random.default_rng(5).random((6, 8)).astype(np.float32) * 6.28
    got, _, _ = odm.generate(img, depth, p, phase=phase)
    ref = _loop_reference(img, depth, p, phase=phase)
    assert np.linalg.norm(got - ref) <= 1e-10 * np.linalg.norm(ref)


def test_oracle_reference_mode_transform():
    img, depth = _tiny(4, 6, 8)
    p = odm.DMParams(pnx=8, pny=6, num_of_depth=3, pad=1, near=0.2, far=0.7, transform_viewing_window=1,
                     rand_phase=cmath.exp(0.7j))
    got, _, _ = odm.generate(img, depth, p)
    ref = _loop_reference(img, depth, p)
    assert np.linalg.norm(got - ref) <= 1e-10 * np.linalg.norm(ref)


def test_centred_fft_matches_dft():
    a = (np.random.default_rng(1).standard_normal((6, 10)) + 1j * np.random.default_rng(2).standard_normal((6, 10)))
    got = odm.centred_fft2(a)
    ref = np.array(_fftshift_cpu(10, 6, _dft2(_fftshift_cpu(10, 6, a.tolist()), -1)))
    assert np.allclose(got, ref, rtol=0, atol=1e-10)


def test_depth_levels_repeated_addition_quirk():
    # 0.30..0.35 in 16 levels: repeated addition stops one short of far
    p = odm.DMParams(num_of_depth=16)
    dstep, lv = odm.depth_levels(p)
    assert len(lv) == 16
    v, n = p.near, 0
    while v <= p.far:
        v += dstep
        n += 1
    assert n == 15                      # the reference's own loop count
    # the 32-level workload is not affected
    _, lv32 = odm.depth_levels(odm.DMParams(num_of_depth=32))
    assert len(lv32) == 32 and abs(lv32[-1] - 0.35) < 1e-12


def test_depth_lut_bins_config():
    lut = odm.depth_lut(odm.DMParams(num_of_depth=32))
    assert lut.min() >= 1 and lut.max() <= 32
    assert lut[255] == 1 and lut[0] == 32        # near plane is depth byte 255
    assert np.all(np.diff(lut) <= 0)
    lut0 = odm.depth_lut(odm.DMParams(flag_change_depth_quantization=0, num_of_depth=256))
    assert np.array_equal(lut0, 256 - np.arange(256))


def test_crop_window_reference_values():
    # Encoding_Symmetrization with sig_location (0,1) on 1920x1080 / 3840x2160
    assert odm.crop_window(1920, 1080, (0, 1)) == (0, 1919, 269, 808)
    assert odm.crop_window(3840, 2160, (0, 1)) == (0, 3839, 539, 1618)
    assert odm.crop_window(1920, 1080, (1, 0)) == (479, 1438, 0, 1079)


def test_library_levels_match_oracle(lib_built):
    """oh_depthmap_levels (host code of the library) bins exactly like the oracle."""
    from openholo_gb300 import depthmap as dm
    for kw in [dict(num_of_depth=32), dict(num_of_depth=16), dict(num_of_depth=256, near=0.2, far=0.7),
               dict(num_of_depth=7, near=0.7, far=0.2), dict(flag_change_depth_quantization=0, num_of_depth=256),
               dict(num_of_depth=1)]:
        p = dm.make_params(**kw)
        lut, z = dm.levels(p)
        op = odm.DMParams(num_of_depth=kw.get("num_of_depth", 32), near=kw.get("near", 0.3), far=kw.get("far", 0.35),
                          flag_change_depth_quantization=kw.get("flag_change_depth_quantization", 1))
        olut = odm.depth_lut(op)
        olut = np.where((olut >= 1) & (olut <= 32767), olut, 0)
        assert np.array_equal(lut.astype(np.int64), olut), kw
        assert np.allclose(z, odm.transformed_levels(op), rtol=0, atol=0), kw


def test_library_levels_transform(lib_built):
    from openholo_gb300 import depthmap as dm
    p = dm.make_params(num_of_depth=8, near=0.2, far=0.7, transform_viewing_window=1, field_lens=1.0)
    _, z = dm.levels(p)
    op = odm.DMParams(num_of_depth=8, near=0.2, far=0.7, transform_viewing_window=1, field_lens=1.0)
    assert np.array_equal(z, np.array(odm.transformed_levels(op)))


def test_as_bandlimited_oracle_limits():
    """The band-limited AS restatement: z -> 0 returns the input (the kernel is
    1 inside the band); a plane wave along the axis keeps its amplitude."""
    from oracle import propagation as oprop
    rng = np.random.default_rng(3)
    U = rng.standard_normal((24, 30)) + 1j * rng.standard_normal((24, 30))
    out = oprop.as_bandlimited(U, 8e-6, 8e-6, 0.0, 532e-9)
    assert np.abs(out - U).max() < 1e-12 * np.abs(U).max()
    plane = np.ones((32, 32), np.complex128)
    out = oprop.as_bandlimited(plane, 8e-6, 8e-6, 1e-3, 532e-9)
    assert abs(abs(out[16, 16]) - 1.0) < 0.05
