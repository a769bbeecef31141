"""CPU oracle for the triangle-mesh CGH (MeshCGH) — TEST INFRASTRUCTURE ONLY.

Restates OpenHolo_MeshCGH in numpy FP64: fn_genH.m:1-53 (frequency grid,
sum of the triangles' angular spectra, fftshift(fft2(fftshift(.)))),
fn_AS_shading.m (flat shading) and fn_AS_continuous.m (continuous shading
with fn_FindVertexNormalVector.m), formula for formula, including the
special-case assignments in the same order.  Two choices that make the
restatement and the GPU path agree bit for bit on the special cases, with
the reason:
  - inv(A') is the closed-form 2x2 inverse (MATLAB's inv may differ in the
    last bit);
  - the face normals of fn_FindVertexNormalVector are not divided by
    norm(no) (a positive scale of all of them; every later use depends only
    on directions).
Parity unpinned (no MATLAB here).
"""
from __future__ import annotations

import math

import numpy as np

REF = np.array([[0.0, 0.0], [1.0, 1.0], [1.0, 0.0]])


def freq_grid(nx, ny, dx, dy, lam):
    dfx = 1.0 / dx / nx
    dfy = 1.0 / dy / ny
    fx = -(np.arange(nx) - nx / 2) * dfx
    fy = (np.arange(ny) - ny / 2) * dfy
    fx, fy = np.meshgrid(fx, fy)
    fz = np.sqrt(((1.0 / lam) ** 2 - fx ** 2 - fy ** 2).astype(np.complex128))
    return fx, fy, fz


def vertex_normals(obj):
    """fn_FindVertexNormalVector: face normals (unnormalised, see module note)
    and per-vertex averages of the face normals of all triangles sharing the
    exact vertex; a vertex at the origin keeps a zero normal (the source
    marks visited rows by zeroing them)."""
    obj = np.asarray(obj, dtype=np.float64)
    T = obj.shape[0]
    na = np.cross(obj[:, 0:3] - obj[:, 3:6], obj[:, 6:9] - obj[:, 3:6])
    objv = obj.reshape(T * 3, 3).copy()
    nv = np.zeros_like(objv)
    for i in range(objv.shape[0]):
        if np.all(objv[i] == 0):
            continue
        idx = np.nonzero(np.all(objv == objv[i], axis=1))[0]
        s = np.zeros(3)
        for j in idx:
            s = s + na[j // 3]
            objv[j] = 0
        avg = s / len(idx)
        avg = avg / np.linalg.norm(avg)
        nv[idx] = avg
    return na, nv.reshape(T, 9)


def _setup(X, n):
    """Rotation, local shift and the reference-triangle map, or None."""
    th = 0.0 if (n[0] == 0 and n[2] == 0) else math.atan(n[0] / n[2])
    ph = math.atan(n[1] / math.sqrt(n[0] ** 2 + n[2] ** 2))
    R = np.array([[math.cos(th), 0.0, -math.sin(th)],
                  [-math.sin(ph) * math.sin(th), math.cos(ph), -math.cos(th) * math.sin(ph)],
                  [math.cos(ph) * math.sin(th), math.sin(ph), math.cos(ph) * math.cos(th)]])
    Xl = R @ X
    c = -Xl[:, 0]
    Xl = Xl + c[:, None]
    if Xl[0, 2] * Xl[1, 1] == Xl[1, 2] * Xl[0, 1]:
        return None
    Xld = Xl[0:2, :].T
    b = Xld[2, 0] * Xld[1, 1] - Xld[2, 1] * Xld[1, 0]
    A = np.zeros((2, 2))
    for l in range(2):
        for m in range(2):
            A[l, m] = (REF[2, l] * Xld[1, 1 - m] - REF[1, l] * Xld[2, 1 - m]) / (b * (-1) ** (m + 2))
    At = A.T
    det = At[0, 0] * At[1, 1] - At[0, 1] * At[1, 0]
    tA = np.array([[At[1, 1], -At[0, 1]], [-At[1, 0], At[0, 0]]]) / det
    return R, c, A, tA


def _local(R, fx, fy, fz, w):
    flx = R[0, 0] * fx + R[0, 1] * fy + R[0, 2] * fz
    fly = R[1, 0] * fx + R[1, 1] * fy + R[1, 2] * fz
    flz = np.sqrt(((1.0 / w) ** 2 - flx ** 2 - fly ** 2).astype(np.complex128))
    return flx, fly, flz


def _G0_flat(fa, fb):
    tp = 2 * np.pi
    with np.errstate(divide="ignore", invalid="ignore"):
        G0 = (np.exp(-1j * tp * fa) - 1) / (tp ** 2 * fa * fb) + (1 - np.exp(-1j * tp * (fa + fb))) / (tp ** 2 * fb * (fa + fb))
        m = (fa == 0) & (fb != 0)
        G0[m] = (1 - np.exp(-1j * tp * fb[m])) / (tp * fb[m]) ** 2 - 1j / (tp * fb[m])
        m = (fa != 0) & (fb == 0)
        G0[m] = (np.exp(-1j * tp * fa[m]) - 1) / (tp * fa[m]) ** 2 + 1j * np.exp(-1j * tp * fa[m]) / (tp * fa[m])
        G0[(fa == fb) & (fa == 0)] = 0.5
        m = (fa == -fb) & (fb != 0)
        G0[m] = (1 - np.exp(1j * tp * fb[m])) / (tp * fb[m]) ** 2 + 1j / (tp * fb[m])
    return G0


def _G0_cont(fa, fb, a1, a2, a3):
    p = np.pi
    e_ab = np.exp(-1j * 2 * p * (fa + fb))
    e_a = np.exp(-1j * 2 * p * fa)
    e_b = np.exp(-1j * 2 * p * fb)
    with np.errstate(divide="ignore", invalid="ignore"):
        D1 = (e_ab * (1j - 2 * p * (fa + fb)) / (8 * p ** 3 * fb * (fa + fb) ** 2)
              + e_a * (2 * p * fa - 1j) / (8 * p ** 3 * fa ** 2 * fb)
              + 1j * (2 * fa + fb) / (8 * p ** 3 * fa ** 2 * (fa + fb) ** 2))
        D2 = (e_ab * (1j * (fa + 2 * fb) - 2 * p * fb * (fa + fb)) / (8 * p ** 3 * fb ** 2 * (fa + fb) ** 2)
              + e_a * (-1j) / (8 * p ** 3 * fa * fb ** 2)
              + 1j / (8 * p ** 3 * fa * (fa + fb) ** 2))
        D3 = (-e_ab / (4 * p ** 2 * fb * (fa + fb))
              + e_a / (4 * p ** 2 * fa * fb)
              - 1 / (4 * p ** 2 * fa * (fa + fb)))
        m = fa == -fb
        x = fa[m]
        ex = np.exp(-1j * 2 * p * x)
        D1[m] = (-2 * p * x + 1j) / (8 * p ** 3 * x ** 3) * ex - (1j * 2 * p ** 2 * x ** 2 + 1j) / (8 * p ** 3 * x ** 3)
        D2[m] = (-1j) / (8 * p ** 3 * x ** 3) * ex + (-1j * 2 * p ** 2 * x ** 2 + 1j + 2 * p * x) / (8 * p ** 3 * x ** 3)
        D3[m] = (-1j) / (4 * p ** 2 * x ** 2) * ex + (-1j * 2 * p * x + 1) / (4 * p ** 2 * x ** 2)
        m = (fa != 0) & (fb == 0)
        x = fa[m]
        ex = np.exp(-1j * 2 * p * x)
        D1[m] = (1j * 4 * p ** 2 * x ** 2 + 4 * p * x - 2 * 1j) / (8 * p ** 3 * x ** 3) * ex + 1j / (4 * p ** 3 * x ** 3)
        D2[m] = 0.5 * D1[m]
        D3[m] = ((1j * 2 * p * x + 1) * ex - 1) / (4 * p ** 2 * x ** 2)
        m = (fa == 0) & (fb != 0)
        y = fb[m]
        ey = np.exp(-1j * 2 * p * y)
        D1[m] = -(2 * p * y + 1) * ey / (8 * p ** 3 * y ** 3) + (-1j * 2 * p ** 2 * y ** 2 + 1) / (8 * p ** 3 * y ** 3)
        D2[m] = (-p * y + 1j) / (4 * p ** 3 * y ** 3) * ey - (1j + p * y) / (4 * p ** 3 * y ** 3)
        D3[m] = ey / (2 * p * y) + (1 - 1j) / (2 * p * y)
        m = (fa == 0) & (fb == 0)
        D1[m] = 1 / 3
        D2[m] = 1 / 6
        D3[m] = 1 / 2
    del e_b
    return (a2 - a1) * D1 + (a3 - a2) * D2 + a1 * D3


def triangle_spectrum(X, fx, fy, fz, w, illu, continuous=False, n_face=None, nv_row=None):
    """fn_AS_shading (continuous=False) or fn_AS_continuous for one triangle
    X (3x3, columns = vertices)."""
    if continuous:
        n = np.asarray(n_face, dtype=np.float64)
    else:
        no = np.cross(X[:, 1] - X[:, 2], X[:, 0] - X[:, 2])
        n = no
    if not n[2] > 0:
        return 0.0
    if not continuous:
        n = n / np.linalg.norm(n)
    st = _setup(X, n)
    if st is None:
        return 0.0
    R, c, A, tA = st
    flx, fly, flz = _local(R, fx, fy, fz, w)
    du = (1.0 / w) * np.array([R[0, 2], R[1, 2]])
    flux = flx - du[0]
    fluy = fly - du[1]
    fa = tA[0, 0] * flux + tA[0, 1] * fluy
    fb = tA[1, 0] * flux + tA[1, 1] * fluy
    if continuous:
        av = np.zeros(3)
        for k in range(3):
            av[k] = nv_row[3 * k] * illu[0] + nv_row[3 * k + 1] * illu[1] + nv_row[3 * k + 2] * illu[2] + 0.1
            if av[k] < 0:
                av[k] = 0
        G0 = _G0_cont(fa, fb, av[0], av[2], av[1])
    else:
        G0 = _G0_flat(fa, fb)
    J = 1.0 / (A[0, 0] * A[1, 1] - A[0, 1] * A[1, 0])
    Gl = J * G0 * np.exp(-1j * 2 * np.pi / w * (R.T @ c)[2])
    G = Gl * (flz / fz) * np.exp(1j * 2 * np.pi * (flx * c[0] + fly * c[1] + flz * c[2]))
    if not continuous:
        if np.all(np.asarray(illu) == 0):
            s = 1.0
        else:
            il = np.asarray(illu, dtype=np.float64) / np.linalg.norm(illu)
            s = max(0.0, n[0] * il[0] + n[1] * il[1] + n[2] * il[2])
        G = G * (2 * s + 0.1)
    return G


def gen_hologram(obj, nx, ny, dx, dy, lam, illu=(1.0, 1.0, 1.0), continuous=False, return_spectrum=False):
    """fn_genH: obj rows (x1 y1 z1 x2 y2 z2 x3 y3 z3)."""
    obj = np.asarray(obj, dtype=np.float64)
    fx, fy, fz = freq_grid(nx, ny, dx, dy, lam)
    GG = np.zeros((ny, nx), np.complex128)
    na = nv = None
    if continuous:
        na, nv = vertex_normals(obj)
    for i in range(obj.shape[0]):
        X = obj[i].reshape(3, 3).T
        G = triangle_spectrum(X, fx, fy, fz, lam, illu, continuous, None if na is None else na[i],
                              None if nv is None else nv[i])
        GG = GG + G
    field = np.fft.fftshift(np.fft.fft2(np.fft.fftshift(GG)))
    return (field, GG) if return_spectrum else field


def ill_conditioned(obj, nx, ny, dx, dy, lam, continuous=False, thresh=1e-3):
    """Samples where some front-facing triangle's reference-triangle
    frequencies (flxA, flyA) come within `thresh` of the source's removable
    singularities (flxA, flyA or flxA + flyA near 0, without being exactly 0).
    There the source's formulas cancel at order 1/f (flat) or 1/f^2
    (continuous), so any double evaluation carries rounding noise ~eps/f^2."""
    obj = np.asarray(obj, dtype=np.float64)
    fx, fy, fz = freq_grid(nx, ny, dx, dy, lam)
    bad = np.zeros((ny, nx), bool)
    na = None
    if continuous:
        na, _ = vertex_normals(obj)
    for i in range(obj.shape[0]):
        X = obj[i].reshape(3, 3).T
        if continuous:
            n = na[i]
        else:
            n = np.cross(X[:, 1] - X[:, 2], X[:, 0] - X[:, 2])
        if not n[2] > 0:
            continue
        if not continuous:
            n = n / np.linalg.norm(n)
        st = _setup(X, n)
        if st is None:
            continue
        R, c, A, tA = st
        flx, fly, _ = _local(R, fx, fy, fz, lam)
        flux = (flx - (1.0 / lam) * R[0, 2]).real
        fluy = (fly - (1.0 / lam) * R[1, 2]).real
        fa = tA[0, 0] * flux + tA[0, 1] * fluy
        fb = tA[1, 0] * flux + tA[1, 1] * fluy
        for v in (fa, fb, fa + fb):
            bad |= (np.abs(v) < thresh) & (v != 0)
    return bad
