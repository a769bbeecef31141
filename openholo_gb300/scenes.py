"""Seeded synthetic inputs for the hologram-generation operators.

The reference ships no usable sample scenes for these shapes (its depth-map
BMPs are not in the tree), so every workload is generated from a seed with a
counter-based SplitMix64 stream: value i of stream s is
splitmix64(seed_s + (i+1)*0x9E3779B97F4A7C15).  Nothing here depends on a
library RNG, so the same seed gives the same scene on every host.
"""
from __future__ import annotations

import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64_at(seed: int, idx: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser applied to seed + (idx+1)*golden (uint64 array)."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + (idx.astype(np.uint64) + np.uint64(1)) * GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n doubles in [0,1) (53 random bits) from stream `stream` of `seed`."""
    s = int(splitmix64_at(seed, np.array([stream], dtype=np.uint64))[0])
    z = splitmix64_at(s, np.arange(n, dtype=np.uint64))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def u24(seed: int, n: int) -> np.ndarray:
    """float32 u in [0,1) with 24 bits, element i from splitmix64_at(seed, i).

    This is the per-pixel phase generator of OH_PHASE_SEEDED."""
    z = splitmix64_at(seed, np.arange(n, dtype=np.uint64))
    return (z >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)


def seeded_phase(seed: int, ny: int, nx: int) -> np.ndarray:
    """Per-pixel phase in radians exactly as the OH_PHASE_SEEDED mode forms it
    (float32 u * float32(2 pi))."""
    return (u24(seed, ny * nx) * np.float32(2.0 * np.pi)).reshape(ny, nx)


def gaussian_sum(seed: int, stream: int, ny: int, nx: int, count: int,
                 sigma_range: tuple[float, float], amp_range=(0.2, 1.0)) -> np.ndarray:
    u = uniform(seed, stream, 4 * count).reshape(count, 4)
    cx = u[:, 0] * nx
    cy = u[:, 1] * ny
    sig = sigma_range[0] + u[:, 2] * (sigma_range[1] - sigma_range[0])
    amp = amp_range[0] + u[:, 3] * (amp_range[1] - amp_range[0])
    x = np.arange(nx, dtype=np.float64)
    y = np.arange(ny, dtype=np.float64)
    out = np.zeros((ny, nx), dtype=np.float64)
    for g in range(count):
        gx = np.exp(-((x - cx[g]) ** 2) / (2 * sig[g] ** 2))
        gy = np.exp(-((y - cy[g]) ** 2) / (2 * sig[g] ** 2))
        out += amp[g] * np.outer(gy, gx)
    return out


def depthmap_scene(seed: int, ny: int = 1080, nx: int = 1920, n_int: int = 20, n_depth: int = 8):
    """uint8 intensity (sum of n_int Gaussians, sigma 20-200 px, rescaled to
    0-255) and uint8 depth (sum of n_depth broad Gaussians rescaled to the
    full 0-255 range).  Sigmas scale with the image size relative to 1080
    rows so that small test frames keep the same structure."""
    scale = min(ny, nx) / 1080.0
    inten = gaussian_sum(seed, 1, ny, nx, n_int, (20 * scale, 200 * scale))
    img = np.clip(np.rint(255.0 * inten / inten.max()), 0, 255).astype(np.uint8)
    dep = gaussian_sum(seed, 2, ny, nx, n_depth, (200 * scale, 600 * scale))
    dep = (dep - dep.min()) / max(dep.max() - dep.min(), 1e-300)
    depth = np.clip(np.rint(255.0 * dep), 0, 255).astype(np.uint8)
    return img, depth


def pointcloud_scene(seed: int, n: int = 5000, xy_half=2e-3, z_range=(0.10, 0.12)):
    """(n,4) float64 x, y, z, amplitude: x,y ~ U(-xy_half, xy_half),
    z ~ U(z_range), a ~ U(0,1)."""
    u = uniform(seed, 3, 4 * n).reshape(n, 4)
    pts = np.empty((n, 4), dtype=np.float64)
    pts[:, 0] = (2 * u[:, 0] - 1) * xy_half
    pts[:, 1] = (2 * u[:, 1] - 1) * xy_half
    pts[:, 2] = z_range[0] + u[:, 2] * (z_range[1] - z_range[0])
    pts[:, 3] = u[:, 3]
    return pts


def wrp_scene(seed: int, n: int = 200_000, box=(10e-3, 10e-3, 2e-3), zc=0.2):
    """(n,3) float64 points uniform in a box centred at (0, 0, zc)."""
    u = uniform(seed, 4, 3 * n).reshape(n, 3)
    pts = np.empty((n, 3), dtype=np.float64)
    pts[:, 0] = (u[:, 0] - 0.5) * box[0]
    pts[:, 1] = (u[:, 1] - 0.5) * box[1]
    pts[:, 2] = zc + (u[:, 2] - 0.5) * box[2]
    return pts


def pls_scene(seed: int, n: int = 5000, xy_half=2e-3, z_range=(0.10, 0.12), amplitude=True):
    """(n, 5) float32 cwoObjPoint records (a_re, a_im, x, y, z): x, y uniform in
    [-xy_half, xy_half), z uniform in z_range, a = |a| e^{i phi} with |a| in
    [0, 1) and phi in [0, 2 pi) (a = 1 when amplitude is False)."""
    u = uniform(seed, 5, 5 * n).reshape(n, 5)
    pts = np.empty((n, 5), dtype=np.float32)
    if amplitude:
        pts[:, 0] = u[:, 0] * np.cos(2 * np.pi * u[:, 1])
        pts[:, 1] = u[:, 0] * np.sin(2 * np.pi * u[:, 1])
    else:
        pts[:, 0], pts[:, 1] = 1.0, 0.0
    pts[:, 2] = (u[:, 2] * 2 - 1) * xy_half
    pts[:, 3] = (u[:, 3] * 2 - 1) * xy_half
    pts[:, 4] = z_range[0] + u[:, 4] * (z_range[1] - z_range[0])
    return pts


def mesh_scene(seed: int, cells: int = 5, size: float = 170e-6, z0: float = 0.1, relief: float = 20e-6,
               back_facing: int = 2):
    """(n, 9) triangles of a seeded height field z = z0 + relief * h(x, y) over
    a cells x cells grid of the given size, two triangles per cell ordered so
    that their normals face +z (shared vertices are bit-identical), followed
    by `back_facing` flipped copies of the first triangles (shifted by `size`
    in x) and one triangle lying in a plane parallel to the hologram."""
    u = uniform(seed, 6, (cells + 1) ** 2).reshape(cells + 1, cells + 1)
    xs = (np.arange(cells + 1) / cells - 0.5) * size
    Z = z0 + relief * (u - 0.5)
    tris = []
    for j in range(cells):
        for i in range(cells):
            a = (xs[i], xs[j], Z[j, i])
            b = (xs[i + 1], xs[j], Z[j, i + 1])
            c = (xs[i], xs[j + 1], Z[j + 1, i])
            d = (xs[i + 1], xs[j + 1], Z[j + 1, i + 1])
            for tri in ((a, c, b), (b, c, d)):
                v1, v2, v3 = (np.array(t) for t in tri)
                if np.cross(v2 - v3, v1 - v3)[2] <= 0:
                    v2, v3 = v3, v2
                tris.append(np.concatenate([v1, v2, v3]))
    for k in range(back_facing):
        # moved off the mesh: a back-facing copy sharing vertices with its
        # original would cancel their averaged normals (0/0 in continuous shading)
        t = tris[k].reshape(3, 3) + np.array([size, 0.0, 0.0])
        tris.append(t[[0, 2, 1]].reshape(-1))
    flat = np.array([[0.0, 0.0, z0], [0.0, 0.3 * size, z0], [0.3 * size, 0.0, z0]])
    if np.cross(flat[1] - flat[2], flat[0] - flat[2])[2] <= 0:
        flat = flat[[0, 2, 1]]
    tris.append(flat.reshape(-1))
    return np.array(tris, dtype=np.float64)


BATCH_FRAMES, BATCH_SEED = 64, 4
BATCH_SCENE_SEED, BATCH_PHASE_SEED = 2024, 77


def batch_workload(n: int = BATCH_FRAMES, seed: int = BATCH_SEED):
    """The mixed depth-map batch: n square frames, side from {512, 768, 1024,
    1536, 2048}, layers 8..64 and wavelength from {450, 532, 633} nm, drawn
    from SplitMix64 stream 9 of `seed`.  Frame i uses the Gaussian scene of
    seed BATCH_SCENE_SEED + side and the seeded per-pixel phase
    BATCH_PHASE_SEED + i; 2x pad, FP32.  Returns [(side, layers, lambda)]."""
    u = uniform(seed, 9, 3 * n).reshape(n, 3)
    sides = [512, 768, 1024, 1536, 2048]
    lams = [450e-9, 532e-9, 633e-9]
    return [(sides[int(a * 5)], 8 + int(b * 57), lams[int(c * 3)]) for a, b, c in u]


def rgbd_scene(seed: int, h: int, w: int) -> np.ndarray:
    """uint8 [h][w][4] RGB-D frame, the float64 twin of oh_scene_rgbd: R, G,
    B = Gaussian sums of streams 3, 1, 5 (20 Gaussians, sigma 20-200 px
    scaled by min(h, w)/1080) each rescaled by its maximum, depth = stream 2
    (8 Gaussians, sigma 200-600 px scaled) rescaled min..max.  G and depth
    equal depthmap_scene(seed, h, w)."""
    scale = min(h, w) / 1080.0
    out = np.empty((h, w, 4), dtype=np.uint8)
    for c, stream in enumerate((3, 1, 5)):
        v = gaussian_sum(seed, stream, h, w, 20, (20 * scale, 200 * scale))
        out[..., c] = np.clip(np.rint(255.0 * v / v.max()), 0, 255).astype(np.uint8)
    d = gaussian_sum(seed, 2, h, w, 8, (200 * scale, 600 * scale))
    d = (d - d.min()) / max(d.max() - d.min(), 1e-300)
    out[..., 3] = np.clip(np.rint(255.0 * d), 0, 255).astype(np.uint8)
    return out
