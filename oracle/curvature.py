"""Curvature frame of a triangle mesh, restated in NumPy (test infrastructure
only): lapy/tria_mesh.py:1078-1279 (curvature, curvature_tria) with its
helpers.  Per-edge dihedral angles accumulated into symmetric 3 x 3 vertex
tensors (Alliez, Cohen-Steiner, Devillers, Levy, Desbrun: Anisotropic
Polygonal Remeshing, 2003), Laplace-smoothed, eigen-decomposed per vertex
with LAPACK (numpy.linalg.eigh, as the reference), pooled to the triangles
and projected into their planes.  The accumulations run in the reference's
order (edges sorted by (i, j)), so the frame equals the reference's to
rounding; tests/test_aniso.py pins it against the reference's outputs.
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




def inner_edges(t, n) -> tuple[np.ndarray, np.ndarray]:
    """Interior edges (i < j, sorted by (i, j)) and, per edge, the triangle
    holding the half-edge i -> j and the one holding j -> i
    (tria_mesh.py:1019-1076 without boundary edges)."""
    m = t.shape[0]
    src = t.reshape(-1)
    dst = t[:, [1, 2, 0]].reshape(-1)
    tri = np.repeat(np.arange(m), 3)
    key = src.astype(np.int64) * n + dst
    order = np.argsort(key, kind="stable")
    skey = key[order]
    fwd = src < dst
    # twin of half-edge (a -> b) is (b -> a)
    twin_key = dst.astype(np.int64) * n + src
    pos = np.searchsorted(skey, twin_key)
    pos_c = np.minimum(pos, len(skey) - 1)
    has_twin = skey[pos_c] == twin_key
    sel = np.nonzero(fwd & has_twin)[0]
    sel = sel[np.argsort(key[sel], kind="stable")]
    vids = np.column_stack((src[sel], dst[sel])).astype(np.int32)
    tids = np.column_stack((tri[sel], tri[order[pos_c[sel]]])).astype(np.int32)
    return vids, tids


def is_oriented(t) -> bool:
    """No directed edge is used twice (tria_mesh.py:604-616)."""
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    return int(np.unique(e, axis=0, return_counts=True)[1].max()) == 1


def curvature(v, t, smoothit: int = 3):
    """Principal directions and curvatures at the vertices
    (tria_mesh.py:1078-1219): u_min, u_max, c_min, c_max, c_mean, c_gauss,
    normals.  The mesh must be oriented."""
    if not is_oriented(t):
        raise ValueError("Error: Can only compute edge information for oriented meshes!")
    n = v.shape[0]
    vids, tids = inner_edges(t, n)
    tn = tria_normals(v, t)
    na, nb = tn[tids[:, 0], :], tn[tids[:, 1], :]
    angle = np.arccos(np.minimum(np.maximum(np.sum(na * nb, axis=1), -1), 1))
    ev = v[vids[:, 1], :] - v[vids[:, 0], :]
    el = np.sqrt(np.sum(ev ** 2, axis=1))
    angle = angle * -np.sign(np.sum(np.cross(na, nb) * ev, axis=1))
    el[el < _EPS] = 1
    ev = ev / el.reshape(-1, 1)
    el = el / np.mean(el)
    # upper triangle of e e' per edge, weighted by the signed angle x length
    ee = np.empty([el.shape[0], 6])
    for c, (a, b) in enumerate(((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))):
        ee[:, c] = ev[:, a] * ev[:, b]
    ee = ee * (angle * el).reshape(-1, 1)
    vv = np.zeros([n, 6])
    np.add.at(vv, vids[:, 0], ee)
    np.add.at(vv, vids[:, 1], ee)
    deg = np.zeros([n])
    np.add.at(deg, vids[:, 0], 1)
    np.add.at(deg, vids[:, 1], 1)
    deg[deg == 0] = 1
    vv = vv / deg.reshape(-1, 1)
    vv = smooth_laplace(v, t, vv, n_iter=smoothit, lambda_=1.0)
    mats = np.empty([n, 3, 3])
    mats[:, 0, :] = vv[:, [0, 1, 2]]
    mats[:, [1, 2], 0] = vv[:, [1, 2]]
    mats[:, 1, [1, 2]] = vv[:, [3, 4]]
    mats[:, 2, 1] = vv[:, 4]
    mats[:, 2, 2] = vv[:, 5]
    evals, evecs = np.linalg.eigh(mats)
    # the eigenvector most aligned with the vertex normal goes first; the
    # other two are the principal directions
    vn = vertex_normals(v, t)
    order = np.argsort(-np.abs(np.squeeze(np.sum(evecs * vn[:, :, np.newaxis], axis=1))), axis=1)
    evals = np.take_along_axis(evals, order, axis=1)
    evecs = np.take_along_axis(evecs, np.tile(order.reshape((n, 1, 3)), (1, 3, 1)), axis=2)
    u_min = np.squeeze(evecs[:, :, 2])
    u_max = np.squeeze(evecs[:, :, 1])
    c_min = evals[:, 1]
    c_max = evals[:, 2]
    normals = np.squeeze(evecs[:, :, 0])
    c_mean = (c_min + c_max) / 2.0
    c_gauss = c_min * c_max
    sw = np.squeeze(np.where(c_min > c_max))
    c_min[sw], c_max[sw] = c_max[sw], c_min[sw]
    u_min[sw, :], u_max[sw, :] = u_max[sw, :], u_min[sw, :]
    normals = normals * np.sign(np.sum(normals * vn, axis=1)).reshape(-1, 1)
    flip = np.squeeze(np.where(np.sum(np.cross(u_min, u_max) * normals, axis=1) < 0))
    u_max[flip, :] = -u_max[flip, :]
    return u_min, u_max, c_min, c_max, c_mean, c_gauss, normals


def curvature_tria(v, t, smoothit: int = 3):
    """Principal directions and curvatures on the triangles
    (tria_mesh.py:1221-1279): vertex values pooled to the triangles, u_min
    projected into the triangle plane and normalised, u_max = n x u_min."""
    u_min, _, c_min, c_max, _, _, _ = curvature(v, t, smoothit)
    tumin = map_vfunc_to_tfunc(t, u_min)
    tcmin = map_vfunc_to_tfunc(t, c_min)
    tcmax = map_vfunc_to_tfunc(t, c_max)
    tn = tria_normals(v, t)
    tumin2 = tumin - tn * (np.sum(tn * tumin, axis=1)).reshape(-1, 1)
    tumin2 = tumin2 / np.maximum(np.sqrt(np.sum(tumin2 * tumin2, axis=1)).reshape(-1, 1), 1e-8)
    return tumin2, np.cross(tn, tumin2), tcmin, tcmax
