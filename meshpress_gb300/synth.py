"""Seeded synthetic meshes for the STRIDE decode workloads.

Every generator is deterministic for a given seed (``numpy.random.default_rng``)
and returns ``(verts float64 (n, 3), tris int64 (m, 3))``.  The shapes follow
the workloads the decoder is measured on:

* ``heightfield_grid`` -- a regular (nx x ny)-vertex grid on the unit square,
  both triangles of every quad cut by the same diagonal ``(a, b, d)/(a, d, c)``,
  heights from seeded sine octaves plus Gaussian noise.  129x129 is the small
  single-mesh case (32,768 triangles); 2049x2049 is the large one (8,388,608).
* ``icosphere`` -- a subdivided icosahedron radially displaced by seeded 3-D
  value noise, with a seeded vertex permutation.  Level 8 has 1,310,720
  triangles.
* ``torus`` -- a (nu x nv) parametric torus.
* ``mixed_batch`` -- many meshes with log-uniform triangle counts, 50 % grids
  of random aspect, 30 % displaced icospheres (levels 3-7), 20 % tori.

The reference's own benchmarks used scanned OBJ meshes that are not part of
the reference repository; these generators stand in for them.
"""
from __future__ import annotations

import math

import numpy as np


# ---------------------------------------------------------------------------
# Heightfields
# ---------------------------------------------------------------------------

def grid_triangles(nx: int, ny: int) -> np.ndarray:
    """Triangles of an nx x ny vertex grid (row-major ids), each quad split
    on the same diagonal: (a, b, d) and (a, d, c) with a=(i,j), b=(i,j+1),
    c=(i+1,j), d=(i+1,j+1)."""
    idx = np.arange(nx * ny, dtype=np.int64).reshape(ny, nx)
    a = idx[:-1, :-1].ravel()
    b = idx[:-1, 1:].ravel()
    c = idx[1:, :-1].ravel()
    d = idx[1:, 1:].ravel()
    t = np.empty((2 * a.size, 3), dtype=np.int64)
    t[0::2] = np.stack([a, b, d], axis=1)
    t[1::2] = np.stack([a, d, c], axis=1)
    return t


def heightfield_grid(n: int = 129, seed: int = 1, *, ny: int | None = None,
                     octaves: int = 4, amplitude: float = 0.1,
                     noise_sigma: float = 0.01,
                     extent: tuple[float, float] = (1.0, 1.0)):
    """Regular heightfield grid with seeded sine-octave heights.

    z = sum_{o<octaves} 2^-o * amplitude * sin(2*pi*2^o*(x cos t_o + y sin t_o) + p_o)
        + N(0, noise_sigma)
    """
    nx = int(n)
    ny = int(ny if ny is not None else n)
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, extent[0], nx)
    ys = np.linspace(0.0, extent[1], ny)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    Z = np.zeros_like(X)
    thetas = rng.uniform(0.0, 2.0 * np.pi, octaves)
    phases = rng.uniform(0.0, 2.0 * np.pi, octaves)
    for o in range(octaves):
        f = 2.0 ** o
        Z += (amplitude / f) * np.sin(
            2.0 * np.pi * f * (X * np.cos(thetas[o]) + Y * np.sin(thetas[o]))
            + phases[o])
    if noise_sigma > 0:
        Z += rng.normal(0.0, noise_sigma, Z.shape)
    V = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    return V, grid_triangles(nx, ny)


def noise_heightfield(n: int = 2049, seed: int = 3, *, octaves: int = 6,
                      base_freq: float = 4.0, amplitude: float = 0.15):
    """Large heightfield with seeded multi-octave 2-D value-noise heights."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, 1.0, n)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    Z = np.zeros_like(X)
    for o in range(octaves):
        f = base_freq * 2.0 ** o
        Z += (amplitude / 2.0 ** o) * _value_noise_2d(X * f, Y * f, rng)
    V = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    return V, grid_triangles(n, n)


def _smooth(t):
    return t * t * (3.0 - 2.0 * t)


def _value_noise_2d(x, y, rng):
    gx = int(np.floor(x.max())) + 2
    gy = int(np.floor(y.max())) + 2
    lat = rng.uniform(-1.0, 1.0, (gy + 1, gx + 1))
    x0 = np.floor(x).astype(np.int64)
    y0 = np.floor(y).astype(np.int64)
    fx = _smooth(x - x0)
    fy = _smooth(y - y0)
    v00 = lat[y0, x0]
    v10 = lat[y0, x0 + 1]
    v01 = lat[y0 + 1, x0]
    v11 = lat[y0 + 1, x0 + 1]
    return (v00 * (1 - fx) + v10 * fx) * (1 - fy) + (v01 * (1 - fx) + v11 * fx) * fy


def _value_noise_3d(p, freq, rng, size=64):
    lat = rng.uniform(-1.0, 1.0, (size, size, size))
    q = (p * freq) % size
    i0 = np.floor(q).astype(np.int64)
    f = _smooth(q - i0)
    i1 = (i0 + 1) % size
    out = np.zeros(len(p))
    for dx in (0, 1):
        wx = f[:, 0] if dx else 1 - f[:, 0]
        ix = i1[:, 0] if dx else i0[:, 0]
        for dy in (0, 1):
            wy = f[:, 1] if dy else 1 - f[:, 1]
            iy = i1[:, 1] if dy else i0[:, 1]
            for dz in (0, 1):
                wz = f[:, 2] if dz else 1 - f[:, 2]
                iz = i1[:, 2] if dz else i0[:, 2]
                out += wx * wy * wz * lat[ix, iy, iz]
    return out


# ---------------------------------------------------------------------------
# Icosphere
# ---------------------------------------------------------------------------

def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    V = np.array([
        [-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
        [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
        [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    F = np.array([
        [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
        [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
        [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
        [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]],
        dtype=np.int64)
    return V / np.linalg.norm(V, axis=1, keepdims=True), F


def _subdivide(V, F):
    """One 4-to-1 midpoint subdivision with shared edge midpoints."""
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    e.sort(axis=1)
    key = e[:, 0] * (len(V) + 1) + e[:, 1]
    uniq, inv = np.unique(key, return_inverse=True)
    a = uniq // (len(V) + 1)
    b = uniq % (len(V) + 1)
    mids = V[a] + V[b]
    mids /= np.linalg.norm(mids, axis=1, keepdims=True)
    mid_id = len(V) + inv
    nf = len(F)
    m01 = mid_id[:nf]
    m12 = mid_id[nf:2 * nf]
    m20 = mid_id[2 * nf:]
    v0, v1, v2 = F[:, 0], F[:, 1], F[:, 2]
    F2 = np.concatenate([
        np.stack([v0, m01, m20], 1), np.stack([v1, m12, m01], 1),
        np.stack([v2, m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return np.concatenate([V, mids]), F2


def icosphere(level: int = 8, seed: int = 2, *, displacement: float = 0.05,
              octaves: int = 5, base_freq: float = 2.0, shuffle: bool = True):
    """Unit icosphere (10*4^L + 2 verts, 20*4^L tris), radially displaced by
    seeded 5-octave 3-D value noise normalised to max |.| = 1 and scaled to
    ``displacement`` of the radius; vertex order permuted by a seeded
    permutation when ``shuffle``."""
    rng = np.random.default_rng(seed)
    V, F = _icosahedron()
    for _ in range(level):
        V, F = _subdivide(V, F)
    if displacement:
        n = np.zeros(len(V))
        for o in range(octaves):
            n += (0.5 ** o) * _value_noise_3d(V + 8.0, base_freq * 2.0 ** o, rng)
        n /= max(np.abs(n).max(), 1e-12)
        V = V * (1.0 + displacement * n)[:, None]
    if shuffle:
        perm = rng.permutation(len(V))
        inv = np.empty_like(perm)
        inv[perm] = np.arange(len(V))
        V = V[perm]
        F = inv[F]
    return V, F


# ---------------------------------------------------------------------------
# Torus
# ---------------------------------------------------------------------------

def torus(nu: int, nv: int, *, R: float = 3.0, r: float = 1.0):
    """Closed parametric torus with nu x nv vertices and 2*nu*nv triangles."""
    u = np.arange(nu) * (2 * np.pi / nu)
    v = np.arange(nv) * (2 * np.pi / nv)
    U, W = np.meshgrid(u, v, indexing="ij")
    X = (R + r * np.cos(W)) * np.cos(U)
    Y = (R + r * np.cos(W)) * np.sin(U)
    Z = r * np.sin(W)
    V = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    i = np.arange(nu)[:, None]
    j = np.arange(nv)[None, :]
    a = (i * nv + j).ravel()
    b = (i * nv + (j + 1) % nv).ravel()
    c = (((i + 1) % nu) * nv + j).ravel()
    d = (((i + 1) % nu) * nv + (j + 1) % nv).ravel()
    F = np.concatenate([np.stack([a, b, d], 1), np.stack([a, d, c], 1)])
    return V, F.astype(np.int64)


# ---------------------------------------------------------------------------
# Mixed batch
# ---------------------------------------------------------------------------

def mixed_batch_specs(n_meshes: int = 4096, seed: int = 4, *,
                      t_min: float = 1e3, t_max: float = 2e5):
    """Seeded list of mesh specs for the many-mesh workload.

    Triangle counts are log-uniform in [t_min, t_max]; kinds are 50 % grids of
    random aspect, 30 % displaced icospheres (level = the one of 3..7 whose
    20*4^L is nearest to the drawn count), 20 % tori (R/r ~ U[2, 5]).
    """
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_meshes):
        t = float(np.exp(rng.uniform(np.log(t_min), np.log(t_max))))
        u = rng.uniform()
        if u < 0.5:
            aspect = float(np.exp(rng.uniform(np.log(0.25), np.log(4.0))))
            quads = max(1.0, t / 2.0)
            w = max(2, int(round(math.sqrt(quads * aspect))) + 1)
            h = max(2, int(round(quads / (w - 1))) + 1)
            specs.append(("grid", dict(nx=w, ny=h, seed=seed * 100003 + i)))
        elif u < 0.8:
            lv = min(range(3, 8), key=lambda L: abs(20 * 4 ** L - t))
            specs.append(("icosphere", dict(level=lv, seed=seed * 100003 + i)))
        else:
            ratio = float(rng.uniform(2.0, 5.0))
            cells = max(9.0, t / 2.0)
            nu = max(3, int(round(math.sqrt(cells * ratio))))
            nv = max(3, int(round(cells / nu)))
            specs.append(("torus", dict(nu=nu, nv=nv, ratio=ratio)))
    return specs


def build_spec(kind: str, params: dict):
    if kind == "grid":
        return heightfield_grid(params["nx"], seed=params["seed"], ny=params["ny"])
    if kind == "icosphere":
        return icosphere(params["level"], seed=params["seed"])
    if kind == "torus":
        return torus(params["nu"], params["nv"], R=params["ratio"], r=1.0)
    raise ValueError(f"unknown mesh kind {kind!r}")


def bbox_bits_error(bits: int) -> float:
    """precision_error for ``precision_mode='bbox_frac'`` that yields ``bits``
    bits on the longest bounding-box axis."""
    return (1.0 + 1e-9) / float((1 << bits) - 1)
