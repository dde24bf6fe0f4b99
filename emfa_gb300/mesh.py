"""Seeded synthetic triangle meshes and the reference's text formats.

The reference reads NASTRAN ``.nas`` meshes (``EMComponent/Mesh.cpp:261-309``):
nine header lines, ``GRID*`` records with a ``*`` continuation line carrying
z, ``CTRIA3`` records and ``ENDDATA``.  Its loader writes every coordinate to a
side file with the default stream precision (6 significant digits) and reads
it back (``Mesh.cpp:291-307,727-779``), so every vertex the reference solves
with is a 6-significant-digit decimal.  The generators here round to the same
grid, so the same mesh reaches the reference, the oracle and the GPU path
bit-identically (float32 for the FP32 path, float64 for the FP64 path).

All meshes are closed, manifold and consistently oriented (counter-clockwise
seen from outside), which is what ``CommonEdge::updateCommonEdge``
(``EMComponent/CommonEdge.cpp:704-743``) needs to pair every edge.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

C0 = 299792458.0  # arma::Datum<float>::c_0 as used by Mathdef.h:28


def round6(a: np.ndarray) -> np.ndarray:
    """Round to 6 significant digits the way ``std::ostream`` (default
    precision, ``%g``) prints a value, then parse back as a double."""
    flat = np.asarray(a, dtype=np.float64).ravel()
    out = np.array([float("%.6g" % v) for v in flat], dtype=np.float64)
    return out.reshape(np.shape(a))


@dataclass
class TriMesh:
    """Vertices (V,3) float64 on the 6-digit grid; triangles (T,3) int32, 0-based."""

    verts: np.ndarray
    tris: np.ndarray
    name: str = "mesh"

    @property
    def n_tri(self) -> int:
        return int(self.tris.shape[0])

    @property
    def n_vert(self) -> int:
        return int(self.verts.shape[0])

    def n_rwg_closed(self) -> int:
        """Interior-edge count of a closed manifold mesh: 3T/2."""
        return 3 * self.n_tri // 2


def _orient_outward(verts: np.ndarray, tris: np.ndarray, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    c = np.asarray(center)
    v0, v1, v2 = verts[tris[:, 0]], verts[tris[:, 1]], verts[tris[:, 2]]
    n = np.cross(v1 - v0, v2 - v0)
    cen = (v0 + v1 + v2) / 3.0 - c
    flip = (n * cen).sum(1) < 0
    out = tris.copy()
    out[flip, 1], out[flip, 2] = tris[flip, 2], tris[flip, 1]
    return out


def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v, f


def icosphere(subdiv: int, radius: float, center=(0.0, 0.0, 0.0)) -> TriMesh:
    """Icosahedron with each triangle split in four ``subdiv`` times, every new
    vertex projected to the sphere.  T = 20*4^s, V = 10*4^s + 2, N = 30*4^s."""
    v, f = _icosahedron()
    verts = [tuple(x) for x in v]
    faces = [tuple(x) for x in f]
    for _ in range(subdiv):
        cache: dict = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key in cache:
                return cache[key]
            p = (np.array(verts[a]) + np.array(verts[b])) * 0.5
            p /= np.linalg.norm(p)
            verts.append(tuple(p))
            cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for (a, b, c) in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    V = np.array(verts) * radius + np.asarray(center)
    T = _orient_outward(V, np.array(faces, dtype=np.int64), center)
    return TriMesh(round6(V), T.astype(np.int32), name=f"icosphere{subdiv}")


def geodesic_sphere(freq: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit sphere: each icosahedron face split into freq^2 triangles on a
    barycentric grid, then projected.  T = 20 f^2, N = 30 f^2."""
    v, f = _icosahedron()
    verts: list = []
    index: dict = {}

    def vid(p):
        key = tuple(np.round(p, 12))
        if key not in index:
            index[key] = len(verts)
            verts.append(p)
        return index[key]

    faces = []
    for (a, b, c) in f:
        A, B, C = v[a], v[b], v[c]
        grid = {}
        for i in range(freq + 1):
            for j in range(freq + 1 - i):
                p = A + (B - A) * (i / freq) + (C - A) * (j / freq)
                p = p / np.linalg.norm(p)
                grid[(i, j)] = vid(p)
        for i in range(freq):
            for j in range(freq - i):
                faces.append((grid[(i, j)], grid[(i + 1, j)], grid[(i, j + 1)]))
                if j + i + 1 < freq:
                    faces.append((grid[(i + 1, j)], grid[(i + 1, j + 1)], grid[(i, j + 1)]))
    V = np.array(verts)
    T = _orient_outward(V, np.array(faces, dtype=np.int64))
    return V, T


def ellipsoid(freq: int, semi_axes, center=(0.0, 0.0, 0.0)) -> TriMesh:
    V, T = geodesic_sphere(freq)
    V = V * np.asarray(semi_axes)[None, :] + np.asarray(center)
    T = _orient_outward(V, T, center)
    return TriMesh(round6(V), T.astype(np.int32), name=f"ellipsoid{freq}")


def cube(m: int, side: float, center=(0.0, 0.0, 0.0)) -> TriMesh:
    """Axis-aligned cube surface, each face an m x m grid of squares split into
    two triangles.  T = 12 m^2, N = 18 m^2."""
    verts: list = []
    index: dict = {}
    h = side / 2.0

    def vid(p):
        key = tuple(int(round(x * 2 * m / side)) for x in p)
        if key not in index:
            index[key] = len(verts)
            verts.append(p)
        return index[key]

    faces = []
    for axis in range(3):
        for s in (-1.0, 1.0):
            u_ax, v_ax = [a for a in range(3) if a != axis]
            for i in range(m):
                for j in range(m):
                    def P(ii, jj):
                        p = [0.0, 0.0, 0.0]
                        p[axis] = s * h
                        p[u_ax] = -h + side * ii / m
                        p[v_ax] = -h + side * jj / m
                        return vid(tuple(p))
                    a, b, c, d = P(i, j), P(i + 1, j), P(i + 1, j + 1), P(i, j + 1)
                    faces.append((a, b, c))
                    faces.append((a, c, d))
    V = np.array(verts) + np.asarray(center)
    T = _orient_outward(V, np.array(faces, dtype=np.int64), center)
    return TriMesh(round6(V), T.astype(np.int32), name=f"cube{m}")


def write_nas(mesh: TriMesh, path: str) -> None:
    """Write the subset of NASTRAN that ``Mesh::loadNasFile`` parses
    (``EMComponent/Mesh.cpp:261-309``)."""
    lines = ["$ emfa_gb300 synthetic mesh", "$", "$", "$", "$", "$", "$", "$",
             "BEGIN BULK"]
    for i, (x, y, z) in enumerate(mesh.verts, start=1):
        lines.append("GRID*   %d %s %s" % (i, "%.6g" % x, "%.6g" % y))
        lines.append("*       %d %s" % (i, "%.6g" % z))
    for i, (a, b, c) in enumerate(mesh.tris, start=1):
        lines.append("CTRIA3  %d 1 %d %d %d" % (i, a + 1, b + 1, c + 1))
    lines.append("ENDDATA")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_nas(path: str) -> TriMesh:
    """Parse the same subset back (used by tests and the launcher front end)."""
    verts, tris = [], []
    with open(path) as f:
        rows = f.read().splitlines()[9:]
    i = 0
    while i < len(rows) and not rows[i].startswith("E"):
        r = rows[i]
        if r.startswith("G"):
            a = r.split("*", 1)[1].split()
            b = rows[i + 1].split("*", 1)[1].split()
            verts.append((float(a[1]), float(a[2]), float(b[1])))
            i += 2
        elif r.startswith("C"):
            a = r.split()[1:]
            tris.append((int(a[2]) - 1, int(a[3]) - 1, int(a[4]) - 1))
            i += 1
        else:
            raise ValueError("unexpected NAS record: %r" % r)
    return TriMesh(round6(np.array(verts)), np.array(tris, dtype=np.int32))


# Every key the reference's ConfigLoader reads on the EFIE/CFIE/MLFMA path
# (EMComponent/ConfigLoader.cpp), with PEC defaults (Sigma zero).
CONFIG_DEFAULTS = {
    "EMSolver:": "EFIE",
    "result_type:": "BistaticRCS",
    "mesh_path:": "mesh.nas",
    "frequency:": "3e8",
    "pole:": "0",
    "frequency_from:": "3e8",
    "frequency_to:": "3e8",
    "frequency_delta:": "3e8",
    "frequency_inc:": "3e8",
    "theta:": "0",
    "phi:": "0",
    "theta_from:": "0",
    "theta_to:": "180",
    "theta_delta:": "1",
    "phi_from:": "0",
    "phi_to:": "0",
    "phi_delta:": "90",
    "E_Plane:": "true",
    "H_Plane:": "true",
    "HH_Plane:": "true",
    "Origin_point:": "(0,0,1)",
    "End_point:": "(3,3,1)",
    "Sampling_x:": "1",
    "Sampling_y:": "1",
    "Sampling_z:": "1",
    "alpha:": "1",
    "preconditioning:": "false",
    "row_threshold:": "0.9",
    "col_threshold:": "0.87",
    "iteration_threshold:": "1e-3",
    "max_iteration_number:": "500",
    "mlfma_box_threshold:": "0.25",
    "thread_number:": "4",
    "task_factor:": "5",
    "Dx:": "0.6",
    "Dy:": "0.6",
    "Array_x:": "20",
    "Array_y:": "20",
    "Sigma:": "(0,0)",
}


def write_config(path: str, **overrides) -> dict:
    """Write a ``CONFIG.yml`` in the reference's ``key: value`` token format
    (``ConfigLoader::load``, ``EMComponent/ConfigLoader.cpp:23-50``)."""
    cfg = dict(CONFIG_DEFAULTS)
    for k, v in overrides.items():
        key = k if k.endswith(":") else k + ":"
        cfg[key] = str(v)
    with open(path, "w") as f:
        f.write("# emfa_gb300 generated config\n")
        for k, v in cfg.items():
            f.write("    %s %s\n" % (k, v))
    return cfg
