"""Seeded synthetic planetary terrain: fBm heightfield plus parabolic craters.

Stands in for the reference's DEM ingest (src/tools/build_from_raster.cu),
which needs GDAL and real rasters.  The mesh follows the raster builder's
rules:
  * cell (cx, cy) with corners v1=(cx,cy), v2=(cx+1,cy), v3=(cx,cy+1),
    v4=(cx+1,cy+1) gives triangles T1=(v1,v3,v2), T2=(v2,v3,v4)
    (build_from_raster.cu:333-360);
  * vertex normals are the incident face normals weighted by the corner
    angle, oriented z-up and normalized (build_from_raster.cu:37-127,388-470).
The grid is centred at the origin with x east, y north (row 0 is north).

Choices the workloads leave open: lacunarity 2, gain 0.5, base wavelength
2560 m; crater count 40 * ((n - 1) / 255)^2 for an n x n grid.
"""
import numpy as np


def _value_noise(rng, nx, ny, spacing, wavelength):
    """Smooth lattice noise in [-1, 1] sampled on an nx x ny grid."""
    cells_x = int(np.ceil((nx - 1) * spacing / wavelength)) + 2
    cells_y = int(np.ceil((ny - 1) * spacing / wavelength)) + 2
    lattice = rng.uniform(-1.0, 1.0, size=(cells_y + 1, cells_x + 1)).astype(np.float32)
    off = rng.uniform(0, 1, size=2)
    gx = (np.arange(nx, dtype=np.float64) * spacing / wavelength + off[0])
    gy = (np.arange(ny, dtype=np.float64) * spacing / wavelength + off[1])
    ix, iy = gx.astype(np.int64), gy.astype(np.int64)
    fx, fy = (gx - ix).astype(np.float32), (gy - iy).astype(np.float32)
    sx = fx * fx * fx * (fx * (fx * 6 - 15) + 10)  # quintic fade
    sy = fy * fy * fy * (fy * (fy * 6 - 15) + 10)
    a = lattice[iy][:, ix]
    b = lattice[iy][:, ix + 1]
    c = lattice[iy + 1][:, ix]
    d = lattice[iy + 1][:, ix + 1]
    top = a + (b - a) * sx[None, :]
    bot = c + (d - c) * sx[None, :]
    return top + (bot - top) * sy[:, None]


def heightfield(n, seed, spacing=10.0, amplitude=200.0, octaves=6, craters=None, base_wavelength=2560.0):
    """n x n heights (float32, metres)."""
    rng = np.random.default_rng(seed)
    h = np.zeros((n, n), np.float32)
    norm = 0.0
    for o in range(octaves):
        g = 0.5 ** o
        h += g * _value_noise(rng, n, n, spacing, base_wavelength / 2 ** o)
        norm += g
    h *= np.float32(amplitude / norm)
    if craters is None:
        craters = int(round(40 * ((n - 1) / 255.0) ** 2))
    extent = (n - 1) * spacing
    for _ in range(craters):
        r = rng.uniform(20.0, 300.0)
        depth = 0.2 * 2 * r
        cx, cy = rng.uniform(0, extent, size=2)
        x0, x1 = max(0, int((cx - r) / spacing)), min(n - 1, int((cx + r) / spacing) + 1)
        y0, y1 = max(0, int((cy - r) / spacing)), min(n - 1, int((cy + r) / spacing) + 1)
        if x1 < x0 or y1 < y0:
            continue
        xs = np.arange(x0, x1 + 1) * spacing - cx
        ys = np.arange(y0, y1 + 1) * spacing - cy
        d2 = (xs[None, :] ** 2 + ys[:, None] ** 2) / (r * r)
        bowl = np.where(d2 < 1.0, depth * (1.0 - d2), 0.0).astype(np.float32)  # parabolic
        h[y0:y1 + 1, x0:x1 + 1] -= bowl
    return h


def mesh_from_heightfield(h, spacing=10.0):
    """Vertices (V x 3 float32), normals (V x 3 float32), indices (M x 3 uint32)."""
    ny, nx = h.shape
    xs = (np.arange(nx, dtype=np.float64) - (nx - 1) / 2.0) * spacing
    ys = ((ny - 1) / 2.0 - np.arange(ny, dtype=np.float64)) * spacing
    V = np.empty((ny, nx, 3), np.float32)
    V[..., 0] = xs[None, :]
    V[..., 1] = ys[:, None]
    V[..., 2] = h
    idx = np.arange(nx * ny, dtype=np.uint32).reshape(ny, nx)
    v1, v2, v3, v4 = idx[:-1, :-1], idx[:-1, 1:], idx[1:, :-1], idx[1:, 1:]
    tris = np.empty((ny - 1, nx - 1, 2, 3), np.uint32)
    tris[:, :, 0] = np.stack([v1, v3, v2], -1)
    tris[:, :, 1] = np.stack([v2, v3, v4], -1)
    I = tris.reshape(-1, 3)
    N = _angle_weighted_normals(V, nx, ny)
    return V.reshape(-1, 3), N.reshape(-1, 3), I


def _angle_weighted_normals(V, nx, ny):
    P = V.astype(np.float32)
    acc = np.zeros_like(P)
    c1, c2, c3, c4 = P[:-1, :-1], P[:-1, 1:], P[1:, :-1], P[1:, 1:]

    def accumulate(a, b, c, sa, sb, sc):
        fn = np.cross(b - a, c - a)
        ln = np.linalg.norm(fn, axis=-1, keepdims=True)
        fn = np.where(ln > 1e-12, fn / np.maximum(ln, 1e-30), 0.0)
        fn = np.where(fn[..., 2:3] < 0, -fn, fn)  # planar z-up orientation

        def corner(p, q, r):
            e1, e2 = q - p, r - p
            e1 = e1 / np.maximum(np.linalg.norm(e1, axis=-1, keepdims=True), 1e-30)
            e2 = e2 / np.maximum(np.linalg.norm(e2, axis=-1, keepdims=True), 1e-30)
            return np.arccos(np.clip((e1 * e2).sum(-1, keepdims=True), -1.0, 1.0))

        acc[sa] += fn * corner(a, b, c)
        acc[sb] += fn * corner(b, c, a)
        acc[sc] += fn * corner(c, a, b)

    s1 = (slice(0, ny - 1), slice(0, nx - 1))
    s2 = (slice(0, ny - 1), slice(1, nx))
    s3 = (slice(1, ny), slice(0, nx - 1))
    s4 = (slice(1, ny), slice(1, nx))
    accumulate(c1, c3, c2, s1, s3, s2)  # T1 = v1, v3, v2
    accumulate(c2, c3, c4, s2, s3, s4)  # T2 = v2, v3, v4
    ln = np.linalg.norm(acc, axis=-1, keepdims=True)
    return np.where(ln > 1e-12, acc / np.maximum(ln, 1e-30), 0.0).astype(np.float32)


def terrain_mesh(n, seed, spacing=10.0, **kw):
    return mesh_from_heightfield(heightfield(n, seed, spacing=spacing, **kw), spacing)
