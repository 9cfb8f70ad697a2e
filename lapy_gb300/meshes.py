"""Deterministic synthetic meshes for tests and benchmarks.

* ``icosahedron()`` / ``icosphere(level)``: midpoint subdivision of a regular
  icosahedron (``TriaMesh.refine_``), every level projected to the unit sphere;
  level L has 10*4^L + 2 vertices and 20*4^L triangles.
* ``sh_deform(mesh, seed)``: radius r = 1 + amp * sum_{l<=lmax, m} c_lm Y_lm with
  real spherical harmonics and c_lm ~ N(0, 1) / (1 + l).
* ``kuhn_cube(n, jitter, seed)``: the unit cube cut into n^3 cells, each into the
  6 Kuhn tetrahedra (monotone lattice paths from corner 000 to 111), interior
  vertices jittered uniformly by +-jitter*h per coordinate.
* ``square_grid(n)`` / ``cube_surface(n)``: planar and closed test meshes.
"""

from __future__ import annotations

import itertools
import math

import numpy as np
from scipy.special import lpmv

from .tet_mesh import TetMesh
from .tria_mesh import TriaMesh


def icosahedron() -> TriaMesh:
    """Regular icosahedron on the unit sphere, outward-oriented faces."""
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    v = []
    for a, b in itertools.product((-1.0, 1.0), repeat=2):
        v += [(0.0, a, b * phi), (a, b * phi, 0.0), (b * phi, 0.0, a)]
    v = np.array(v)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    d = np.linalg.norm(v[:, None, :] - v[None, :, :], axis=2)
    edge = d[d > 1e-9].min()
    adj = np.abs(d - edge) < 1e-9
    faces = []
    for i, j, k in itertools.combinations(range(12), 3):
        if adj[i, j] and adj[j, k] and adj[i, k]:
            nrm = np.cross(v[j] - v[i], v[k] - v[i])
            faces.append((i, j, k) if nrm @ (v[i] + v[j] + v[k]) > 0 else (i, k, j))
    return TriaMesh(v, np.array(faces, dtype=np.int64))


def icosphere(level: int) -> TriaMesh:
    """Unit icosphere: ``level`` midpoint subdivisions, each projected to r = 1."""
    T = icosahedron()
    for _ in range(level):
        T.refine_()
        T = TriaMesh(T.v / np.linalg.norm(T.v, axis=1, keepdims=True), T.t)
    return T


def real_sph_harm(l: int, m: int, theta: np.ndarray, phi: np.ndarray) -> np.ndarray:
    """Orthonormal real spherical harmonic Y_lm (theta: polar, phi: azimuth)."""
    am = abs(m)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    p = lpmv(am, l, np.cos(theta))
    if m == 0:
        return norm * p
    if m > 0:
        return math.sqrt(2.0) * norm * p * np.cos(am * phi)
    return math.sqrt(2.0) * norm * p * np.sin(am * phi)


def sh_deform(mesh: TriaMesh, seed: int, lmax: int = 8, amp: float = 0.1) -> TriaMesh:
    """Radial spherical-harmonic deformation of a unit-sphere mesh."""
    rng = np.random.default_rng(seed)
    v = np.asarray(mesh.v, dtype=np.float64)
    u = v / np.linalg.norm(v, axis=1, keepdims=True)
    theta = np.arccos(np.clip(u[:, 2], -1.0, 1.0))
    phi = np.arctan2(u[:, 1], u[:, 0])
    r = np.ones(len(v))
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            c = rng.standard_normal() / (1.0 + l)
            r += amp * c * real_sph_harm(l, m, theta, phi)
    return TriaMesh(u * r[:, None], mesh.t.copy())


def deformed_icospheres(levels, seeds, lmax: int = 8, amp: float = 0.1) -> list:
    """``sh_deform(icosphere(level), seed)`` for many meshes, with the icosphere
    and its spherical-harmonic basis built once per level."""
    base, basis = {}, {}
    out = []
    for level, seed in zip(levels, seeds):
        level = int(level)
        if level not in base:
            m = icosphere(level)
            u = m.v / np.linalg.norm(m.v, axis=1, keepdims=True)
            th = np.arccos(np.clip(u[:, 2], -1.0, 1.0))
            ph = np.arctan2(u[:, 1], u[:, 0])
            base[level] = (m, u)
            basis[level] = np.stack([real_sph_harm(l, mm, th, ph) for l in range(lmax + 1)
                                     for mm in range(-l, l + 1)], axis=1)
        m, u = base[level]
        scale = np.array([1.0 / (1 + l) for l in range(lmax + 1) for _ in range(2 * l + 1)])
        c = np.random.default_rng(int(seed)).standard_normal(len(scale)) * scale
        r = 1.0 + amp * (basis[level] @ c)
        out.append(TriaMesh(u * r[:, None], m.t.copy()))
    return out


def kuhn_cube(n: int, jitter: float = 0.0, seed: int = 0) -> TetMesh:
    """Unit cube, n^3 cells x 6 Kuhn tetrahedra; vertex (i,j,k) has index i + (n+1)(j + (n+1)k)."""
    h = 1.0 / n
    g = np.arange(n + 1) * h
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    v = np.column_stack((x.ravel(), y.ravel(), z.ravel()))
    if jitter:
        rng = np.random.default_rng(seed)
        idx = np.arange(n + 1)
        kk, jj, ii = np.meshgrid(idx, idx, idx, indexing="ij")
        interior = ((ii > 0) & (ii < n) & (jj > 0) & (jj < n) & (kk > 0) & (kk < n)).ravel()
        v[interior] += rng.uniform(-jitter * h, jitter * h, size=(int(interior.sum()), 3))
    s = n + 1
    ci, cj, ck = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = (ci + s * (cj + s * ck)).transpose(2, 1, 0).ravel()
    step = np.array([1, s, s * s])
    tets = []
    for perm in itertools.permutations(range(3)):
        a = base
        b = a + step[perm[0]]
        c = b + step[perm[1]]
        d = c + step[perm[2]]
        tets.append(np.column_stack((a, b, c, d)))
    t = np.stack(tets, axis=1).reshape(-1, 4)
    return TetMesh(v, t)


def kuhn_center_vertex(n: int) -> int:
    c = n // 2
    return c + (n + 1) * (c + (n + 1) * c)


def square_grid(n: int) -> TriaMesh:
    """Unit square, n x n cells, each split into 2 triangles."""
    g = np.linspace(0.0, 1.0, n + 1)
    y, x = np.meshgrid(g, g, indexing="ij")
    v = np.column_stack((x.ravel(), y.ravel(), np.zeros(x.size)))
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = (i * (n + 1) + j).ravel()
    b, c, d = a + 1, a + n + 1, a + n + 2
    t = np.column_stack((a, b, d, a, d, c)).reshape(-1, 3)
    return TriaMesh(v, t)


def cube_surface(n: int) -> TriaMesh:
    """Closed surface of the unit cube, n x n cells per face, 2 triangles each."""
    verts = {}
    vlist = []

    def vid(p):
        key = tuple(np.round(np.asarray(p) * n).astype(int))
        if key not in verts:
            verts[key] = len(vlist)
            vlist.append(np.asarray(key, dtype=np.float64) / n)
        return verts[key]

    tris = []
    g = np.arange(n + 1) / n
    for axis in range(3):
        for side in (0.0, 1.0):
            u_ax, w_ax = [a for a in range(3) if a != axis]
            for a in range(n):
                for b in range(n):
                    def P(ua, wb):
                        p = np.zeros(3)
                        p[axis] = side
                        p[u_ax] = g[ua]
                        p[w_ax] = g[wb]
                        return vid(p)
                    p00, p10, p01, p11 = P(a, b), P(a + 1, b), P(a, b + 1), P(a + 1, b + 1)
                    if (side == 1.0) == (axis == 1):
                        tris += [(p00, p11, p10), (p00, p01, p11)]
                    else:
                        tris += [(p00, p10, p11), (p00, p11, p01)]
    return TriaMesh(np.array(vlist), np.array(tris, dtype=np.int64))
