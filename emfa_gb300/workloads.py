"""Seeded synthetic problem sets for the batched and served engines.

batch_set     64 independent EFIE problems of uneven size: PEC ellipsoids
              (semi-axes uniform in 0.3..1.5 wavelengths) and axis-aligned
              cubes meshed at about lambda/10, 500..8000 RWG unknowns,
              f uniform in 200..600 MHz, 8 seeded incidences each with their
              monostatic directions.
served_stream Poisson arrivals (mean 200 requests/s) of monostatic RCS
              requests on spheres, ellipsoids and cubes with unknown counts
              log-uniform in 1k..120k, meshed at about lambda/10 (CFIE,
              alpha 0.5); dense below 10k unknowns, MLFMA above.

No public dataset is involved: every mesh is generated here from the seed.
"""
from __future__ import annotations

import math

import numpy as np

from . import mesh as M

C0 = 299792458.0


def geodesic_sphere_fast(freq: int):
    """Unit sphere with T = 20 freq^2 triangles (icosahedron faces on a
    barycentric grid, projected), vectorised; vertex order differs from
    mesh.geodesic_sphere."""
    v, f = M._icosahedron()
    ii, jj = np.meshgrid(np.arange(freq + 1), np.arange(freq + 1), indexing="ij")
    keep = (ii + jj) <= freq
    ii, jj = ii[keep], jj[keep]
    gid = -np.ones((freq + 1, freq + 1), dtype=np.int64)
    gid[ii, jj] = np.arange(ii.size)
    # the two triangle families of the barycentric grid
    a_i, a_j = np.nonzero(np.add.outer(np.arange(freq), np.arange(freq)) < freq)
    up = np.stack([gid[a_i, a_j], gid[a_i + 1, a_j], gid[a_i, a_j + 1]], 1)
    b_i, b_j = np.nonzero(np.add.outer(np.arange(freq), np.arange(freq)) + 1 < freq)
    dn = np.stack([gid[b_i + 1, b_j], gid[b_i + 1, b_j + 1], gid[b_i, b_j + 1]], 1)
    loc = np.concatenate([up, dn])
    pts, faces = [], []
    for k, (a, b, c) in enumerate(f):
        A, B, C = v[a], v[b], v[c]
        p = A + np.outer(ii / freq, B - A) + np.outer(jj / freq, C - A)
        pts.append(p / np.linalg.norm(p, axis=1, keepdims=True))
        faces.append(loc + k * ii.size)
    P = np.concatenate(pts)
    F = np.concatenate(faces)
    key = np.round(P, 10)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    V = P[first]
    T = inv.reshape(-1)[F]
    T = M._orient_outward(V, T)
    return V, T


def _ellipsoid_area(a, b, c):
    p = 1.6075
    return 4 * math.pi * ((a ** p * b ** p + a ** p * c ** p + b ** p * c ** p) / 3) ** (1 / p)


def ellipsoid_mesh(semi, lam, n_lo=500, n_hi=8000):
    """Ellipsoid meshed at about lambda/10 (equilateral-triangle estimate),
    the grid clamped so that N = 30 freq^2 stays in [n_lo, n_hi]."""
    h = lam / 10
    T = _ellipsoid_area(*semi) / (math.sqrt(3) / 4 * h * h)
    fq = int(round(math.sqrt(T / 20)))
    fq = max(int(math.ceil(math.sqrt(n_lo / 30))), min(int(math.sqrt(n_hi / 30)), fq))
    V, T = geodesic_sphere_fast(fq)
    V = V * np.asarray(semi)[None, :]
    return M.TriMesh(M.round6(V), M._orient_outward(V, T).astype(np.int32), name=f"ellipsoid_f{fq}")


def batch_set(seed=0, count=64, n_inc=8):
    """The batched set as (mesh, freq Hz, angles (n_inc x 3), monostatic dirs)."""
    from . import api
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        f = float(rng.uniform(200e6, 600e6))
        lam = C0 / f
        if rng.random() < 0.5:
            semi = rng.uniform(0.3, 1.5, 3) * lam
            m = ellipsoid_mesh(semi, lam)
        else:
            side_cells = int(rng.integers(6, 22))  # N = 18 m^2 in 648..7938
            m = M.cube(side_cells, side_cells * lam / 10)
        ang = np.stack([rng.uniform(0, 180, n_inc), rng.uniform(0, 360, n_inc), np.zeros(n_inc)], 1)
        out.append((m, f, ang, api.monostatic_dirs(ang)))
    return out


_cache: dict = {}


def _stream_mesh(shape, n_target, rng):
    if shape == "cube":
        cells = max(8, int(round(math.sqrt(n_target / 18))))
        key = ("cube", cells)
        if key not in _cache:
            _cache[key] = M.cube(cells, 1.0)
        return _cache[key], 1.0 / cells  # grid spacing of the unit cube
    fq = max(6, int(round(math.sqrt(n_target / 30))))
    key = ("sphere", fq)
    if key not in _cache:
        _cache[key] = geodesic_sphere_fast(fq)
    V, T = _cache[key]
    if shape == "ellipsoid":
        semi = np.array([1.0, rng.uniform(0.5, 1.0), rng.uniform(0.5, 1.0)])
        V = V * semi[None, :]
    edge = math.sqrt(4 * math.pi * 4 / (math.sqrt(3) * T.shape[0]))
    return M.TriMesh(M.round6(V), M._orient_outward(V, T).astype(np.int32), name=f"{shape}_f{fq}"), edge


def served_stream(seed=0, count=100, rate=200.0, n_inc=4, n_lo=1000, n_hi=120000):
    """The served stream as (arrival s, mesh, freq Hz, angles, monostatic dirs)."""
    from . import api
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(count):
        t += float(rng.exponential(1.0 / rate))
        n_target = math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))
        shape = ("sphere", "ellipsoid", "cube")[int(rng.integers(0, 3))]
        m, edge = _stream_mesh(shape, n_target, rng)
        f = C0 / (10 * edge)  # lambda/10 mesh
        ang = np.stack([rng.uniform(0, 180, n_inc), rng.uniform(0, 360, n_inc), np.zeros(n_inc)], 1)
        out.append((t, m, f, ang, api.monostatic_dirs(ang)))
    return out
