"""Host mesh utilities of TriaMesh that lie off the FEM path (lapy/tria_mesh.py):
triangle and vertex normals, vertex areas, the 1-ring smoothing matrix and
Laplace smoothing, and triangle means of vertex functions.  The curvature
frame of the anisotropic Laplacian, which uses the same constructions, runs
on the GPU (csrc/curvature.cu).
"""

from __future__ import annotations

import sys

import numpy as np
from scipy import sparse

_EPS = sys.float_info.epsilon


def _corners(v, t):
    return v[t[:, 0], :], v[t[:, 1], :], v[t[:, 2], :]


def tria_normals(v, t) -> np.ndarray:
    """Unit normals (v1 - v0) x (v2 - v0) (tria_mesh.py:750-773)."""
    p0, p1, p2 = _corners(v, t)
    n = np.cross(p1 - p0, p2 - p0)
    ln = np.sqrt(np.sum(n * n, axis=1))
    ln[ln < _EPS] = 1
    return n / ln.reshape(-1, 1)


def vertex_normals(v, t) -> np.ndarray:
    """Sum of the area-weighted normals of the incident triangles, as the
    cross product at each corner (tria_mesh.py:775-817), normalised."""
    p0, p1, p2 = _corners(v, t)
    d10, d21, d02 = p1 - p0, p2 - p1, p0 - p2
    n = np.zeros(v.shape)
    np.add.at(n, t[:, 0], np.cross(d10, -d02))
    np.add.at(n, t[:, 1], np.cross(d21, -d10))
    np.add.at(n, t[:, 2], np.cross(d02, -d21))
    ln = np.sqrt(np.sum(n * n, axis=1))
    ln[ln < _EPS] = 1
    return n / ln.reshape(-1, 1)


def vertex_areas(v, t) -> np.ndarray:
    """One third of the incident triangles' areas (tria_mesh.py:715-733)."""
    p0, p1, p2 = _corners(v, t)
    cr = np.cross(p1 - p0, p2 - p0)
    area = 0.5 * np.sqrt(np.sum(cr * cr, axis=1))
    return np.bincount(t.reshape(-1), np.repeat(area[:, None], 3, 1).reshape(-1)) / 3.0


def adj_sym(t, n) -> sparse.csc_matrix:
    """Symmetric edge-count matrix (entry 2 for an interior edge)."""
    t0, t1, t2 = t[:, 0], t[:, 1], t[:, 2]
    i = np.column_stack((t0, t1, t1, t2, t2, t0)).reshape(-1)
    j = np.column_stack((t1, t0, t2, t1, t0, t2)).reshape(-1)
    return sparse.csc_matrix((np.ones(i.shape), (i, j)), shape=(n, n))


def smoothing_matrix(v, t) -> sparse.csr_matrix:
    """Row-stochastic 1-ring averaging matrix of tria_mesh.py:1696-1715 (each
    row of the binarised adjacency scaled by the row vertex's area, then
    normalised to unit row sum)."""
    n = v.shape[0]
    areas = vertex_areas(v, t)[:, np.newaxis]
    adj = adj_sym(t, n)
    adj.data = np.ones(adj.data.shape)
    adj2 = adj.multiply(areas)
    rowsum = np.sum(adj2, axis=1)
    rowsum[rowsum == 0] = 1.0
    return adj2.multiply(1.0 / rowsum)


def smooth_laplace(v, t, vfunc, n_iter: int = 1, lambda_: float = 0.5, mat=None) -> np.ndarray:
    """n_iter steps of vfunc <- (1 - lambda) vfunc + lambda S vfunc
    (tria_mesh.py:1747-1792)."""
    vfunc = np.array(vfunc)
    if v.shape[0] != vfunc.shape[0]:
        raise ValueError("Error: length of vfunc needs to match number of vertices")
    if mat is None:
        mat = smoothing_matrix(v, t)
    for _ in range(n_iter):
        vfunc = (1.0 - lambda_) * vfunc + lambda_ * mat.dot(vfunc)
    return vfunc


def map_vfunc_to_tfunc(t, vfunc) -> np.ndarray:
    """Mean of a vertex function over each triangle's corners
    (tria_mesh.py:1668-1694)."""
    vfunc = np.array(vfunc) / 3.0
    return np.sum(vfunc[t], axis=1)


