"""NumPy/SciPy restatement of the reference's FEM path (test infrastructure).

Every function cites the reference lines it restates.  Element arithmetic is
performed in the coordinate dtype with NumPy's operation order, so local
element values are bit-identical to the reference's; matrices are summed
either with SciPy's COO->CSC conversion (as the reference does) or in the
deterministic (row, column, element, slot) order the GPU uses.
"""

from __future__ import annotations

import sys

import numpy as np
from scipy import sparse
from scipy.sparse.linalg import LinearOperator, eigsh, splu

EPS = sys.float_info.epsilon

# Local (i, j) slot tables in the reference's COO order.
# triangles: lapy/solver.py:174-175 ; tetrahedra: lapy/solver.py:492-497
TRIA_IJ = (np.array([0, 1, 1, 2, 2, 0, 0, 1, 2]), np.array([1, 0, 2, 1, 0, 2, 0, 1, 2]))
TET_IJ = (np.array([0, 1, 1, 2, 2, 0, 0, 3, 1, 3, 2, 3, 0, 1, 2, 3]),
          np.array([1, 0, 2, 1, 0, 2, 3, 0, 3, 1, 3, 2, 0, 1, 2, 3]))


def _rowdot(a, b):
    """np.sum(a * b, axis=1) for n x 3 arrays: (a0*b0 + a1*b1) + a2*b2."""
    return np.sum(a * b, axis=1)


def _clamp(vol):
    """vol < eps -> max(1e-4 * mean(vol), eps)  (solver.py:158-159, :272-273, :436-437)."""
    vol = vol.copy()
    vm = max(0.0001 * np.mean(vol), EPS)
    vol[vol < EPS] = vm
    return vol


def tria_local(v, t, lump=False, frame=None):
    """Per-triangle local matrices (solver.py:145-193; anisotropic: :248-307).

    Returns (la (m, 9), lm (m, 9) or (m, 3) when lumped), in the coordinate dtype
    (float64 for the anisotropic form, whose frame is float64)."""
    p1, p2, p3 = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    d21, d32, d13 = p2 - p1, p3 - p2, p1 - p3
    cr = np.cross(d32, d13)
    vol = _clamp(2 * np.sqrt(np.sum(cr * cr, axis=1)))
    if frame is None:
        c12, c23, c31 = _rowdot(d32, d13) / vol, _rowdot(d13, d21) / vol, _rowdot(d21, d32) / vol
    else:
        u1, u2, am = frame
        proj = [np.column_stack((np.sum(u1 * d, axis=1), np.sum(u2 * d, axis=1))) for d in (d21, d32, d13)]
        q21, q32, q13 = proj
        c12 = np.sum(q32 * am * q13, axis=1) / vol
        c23 = np.sum(q13 * am * q21, axis=1) / vol
        c31 = np.sum(q21 * am * q32, axis=1) / vol
    la = np.column_stack((c12, c12, c23, c23, c31, c31, -c12 - c31, -c12 - c23, -c31 - c23))
    if lump:
        b = vol / 12
        lm = np.column_stack((b, b, b))
    else:
        bd, bo = vol / 24, vol / 48
        lm = np.column_stack((bo, bo, bo, bo, bo, bo, bd, bd, bd))
    return la, lm


def tet_local(v, t, lump=False):
    """Per-tetrahedron local matrices (solver.py:418-532)."""
    q1, q2, q3, q4 = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]], v[t[:, 3]]
    e1, e2, e3, e4, e5, e6 = q2 - q1, q3 - q2, q1 - q3, q4 - q1, q4 - q2, q4 - q3
    vol = _clamp(np.abs(np.sum(e4 * np.cross(e1, e3), axis=1)))
    dd = {name: _rowdot(a, b) for name, (a, b) in {
        "11": (e1, e1), "22": (e2, e2), "33": (e3, e3), "44": (e4, e4), "55": (e5, e5), "66": (e6, e6),
        "12": (e1, e2), "13": (e1, e3), "14": (e1, e4), "15": (e1, e5), "23": (e2, e3), "25": (e2, e5),
        "26": (e2, e6), "34": (e3, e4), "36": (e3, e6)}.items()}
    # (El.Ek)(Em.Ek) - (El.Em)(Ek.Ek) over the volume (solver.py:460-465)
    a12 = (-dd["36"] * dd["26"] + dd["23"] * dd["66"]) / vol
    a13 = (-dd["15"] * dd["25"] + dd["12"] * dd["55"]) / vol
    a14 = (dd["23"] * dd["26"] - dd["36"] * dd["22"]) / vol
    a23 = (-dd["14"] * dd["34"] + dd["13"] * dd["44"]) / vol
    a24 = (dd["13"] * dd["34"] - dd["14"] * dd["33"]) / vol
    a34 = (-dd["14"] * dd["13"] + dd["11"] * dd["34"]) / vol
    diag = [-a12 - a13 - a14, -a12 - a23 - a24, -a13 - a23 - a34, -a14 - a24 - a34]
    la = np.column_stack((a12, a12, a23, a23, a13, a13, a14, a14, a24, a24, a34, a34, *diag)) / 6.0
    if lump:
        b = vol / 24.0
        lm = np.column_stack((b, b, b, b))
    else:
        bd, bo = vol / 60.0, vol / 120.0
        lm = np.column_stack([bo] * 12 + [bd] * 4)
    return la, lm


def _pairs(t, npe):
    I, J = TRIA_IJ if npe == 3 else TET_IJ
    return t[:, I].reshape(-1), t[:, J].reshape(-1)


def assemble_scipy(v, t, lump=False, dtype=np.float64, frame=None):
    """(A, M) as the reference builds them: csc_matrix((data, (i, j))) (solver.py:178, :187, :501, :526)."""
    npe = t.shape[1]
    la, lm = tria_local(v, t, lump, frame) if npe == 3 else tet_local(v, t, lump)
    i, j = _pairs(t, npe)
    A = sparse.csc_matrix((la.reshape(-1).astype(dtype, copy=False), (i, j)), dtype=dtype)
    if lump:
        d = t.reshape(-1)
        M = sparse.csc_matrix((lm.reshape(-1).astype(dtype, copy=False), (d, d)), dtype=dtype)
    else:
        M = sparse.csc_matrix((lm.reshape(-1).astype(dtype, copy=False), (i, j)), dtype=dtype)
    return A, M


def csr_sorted_sum(i, j, vals, n):
    """CSR with entries summed in (row, col, COO position) order — the GPU's order."""
    pos = np.arange(i.size)
    order = np.lexsort((pos, j, i))
    ii, jj, vv = i[order], j[order], vals[order]
    first = np.ones(ii.size, dtype=bool)
    first[1:] = (ii[1:] != ii[:-1]) | (jj[1:] != jj[:-1])
    starts = np.flatnonzero(first)
    data = np.empty(starts.size, dtype=vals.dtype)
    # sequential sums inside each run (np.add.reduceat sums pairwise for long runs)
    ends = np.append(starts[1:], ii.size)
    maxlen = int((ends - starts).max()) if starts.size else 0
    data[:] = vv[starts]
    for k in range(1, maxlen):
        sel = (starts + k) < ends
        data[sel] = data[sel] + vv[starts[sel] + k]
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(indptr, ii[starts] + 1, 1)
    return sparse.csr_matrix((data, jj[starts], np.cumsum(indptr)), shape=(n, n))


def assemble_sorted(v, t, lump=False, dtype=np.float64, frame=None):
    """(A, M) with the GPU's deterministic summation order; lumped M as an n-vector."""
    npe = t.shape[1]
    n = int(t.max()) + 1
    la, lm = tria_local(v, t, lump, frame) if npe == 3 else tet_local(v, t, lump)
    i, j = _pairs(t, npe)
    A = csr_sorted_sum(i, j, la.reshape(-1).astype(dtype), n)
    if lump:
        d = t.reshape(-1)
        M = csr_sorted_sum(d, d, lm.reshape(-1).astype(dtype), n).diagonal()
    else:
        M = csr_sorted_sum(i, j, lm.reshape(-1).astype(dtype), n)
    return A, M


def avg_edge_length(v, t):
    """Mean length of the distinct edges (tria_mesh.py:735-748, tet_mesh.py:182-195)."""
    npe = t.shape[1]
    i, j = _pairs(t, npe)
    n = v.shape[0]
    adj = sparse.csc_matrix((np.ones(i.size), (i, j)), shape=(n, n))
    up = sparse.triu(adj, 1, format="coo")
    return np.sqrt(((v[up.row] - v[up.col]) ** 2).sum(1)).mean()


def eigs(A, M, k=10, sigma=-0.01, v0=None):
    """Shift-invert eigsh with OPinv = splu(A - sigma M).solve (solver.py:702-716).

    ``v0=None`` is the reference's call.  ARPACK then draws its start vector
    from an internal generator whose state depends on earlier calls in the
    process, and on meshes with exactly degenerate eigenvalues (icospheres) a
    single-vector Krylov space can miss a member of a group; checkers pass a
    seeded ``v0`` or use ``eigs_dense``."""
    lu = splu(sparse.csc_matrix(A - sigma * M))
    op = LinearOperator(matvec=lu.solve, shape=A.shape, dtype=A.dtype)
    return eigsh(A, k, M, sigma=sigma, OPinv=op, v0=v0)


def eigs_dense(A, M, k=10):
    """The k smallest eigenpairs of A x = lambda M x by dense LAPACK (small n)."""
    from scipy.linalg import eigh

    Ad = sparse.csr_matrix(A).toarray()
    Md = sparse.csr_matrix(M).toarray() if sparse.issparse(M) else np.diag(np.asarray(M))
    Ad = 0.5 * (Ad + Ad.T)
    Md = 0.5 * (Md + Md.T)
    return eigh(Ad, Md, subset_by_index=[0, k - 1])


def poisson(A, M, h=0.0, dtup=(), ntup=()):
    """Poisson solve with Dirichlet/Neumann data (solver.py:771-889), via splu."""
    dim = A.shape[0]
    h = np.full((dim, 1), h) if np.isscalar(h) else np.asarray(h, dtype=np.float64)
    if h.ndim == 1:
        h = h[:, None]
    nr = h.shape[1]
    dvec = np.zeros((dim, nr))
    nvec = np.zeros((dim, nr))
    didx = np.asarray(dtup[0]) if dtup else np.array([], dtype=int)
    if dtup:
        dvec[didx, :] = np.asarray(dtup[1])[:, None]
    if ntup:
        np.add.at(nvec, np.asarray(ntup[0]), np.asarray(ntup[1], dtype=np.float64)[:, None])
    b = M @ (h - nvec) - A @ dvec
    if didx.size:
        mask = np.ones(dim, dtype=bool)
        mask[didx] = False
        a = sparse.csc_matrix(A)[:, mask].tocsr()[mask, :].tocsc()
        x = np.zeros((dim, nr))
        x[mask] = splu(a).solve(b[mask])
        x[didx] = dvec[didx]
    else:
        x = splu(sparse.csc_matrix(A)).solve(b)
    return x[:, 0] if nr == 1 else x


def diffusion(v, t, vids, m=1.0):
    """Backward-Euler heat step from seed sets (heat.py:184-232)."""
    if isinstance(vids, list) and vids and isinstance(vids[0], (list, np.ndarray)):
        sets, scalar = [np.asarray(s, dtype=int).ravel() for s in vids], False
    else:
        sets, scalar = [np.asarray(vids, dtype=int).ravel()], True
    A, M = assemble_scipy(v, t, lump=True)
    tt = m * avg_edge_length(v, t) ** 2
    b0 = np.zeros((len(v), len(sets)))
    for c, s in enumerate(sets):
        b0[s, c] = 1.0
    u = splu(sparse.csc_matrix(M + tt * A)).solve(b0)
    return u[:, 0] if scalar else u


def tria_gradient(v, t, f):
    """diffgeo.py:261-298 (1-D or 2-D f)."""
    f = np.asarray(f)
    p0, p1, p2 = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    e2, e0, e1 = p1 - p0, p2 - p1, p0 - p2
    nrm = np.cross(e2, -e1)
    ln = np.sqrt(np.sum(nrm * nrm, axis=1))
    ln[ln < EPS] = 1
    lni = np.divide(1.0, ln)[:, None]
    nrm *= lni
    if f.ndim == 1:
        c = f[t[:, 0], None] * e0 + f[t[:, 1], None] * e1 + f[t[:, 2], None] * e2
        return lni * np.cross(nrm, c)
    c = (f[t[:, 0]][:, :, None] * e0[:, None, :] + f[t[:, 1]][:, :, None] * e1[:, None, :]
         + f[t[:, 2]][:, :, None] * e2[:, None, :])
    return lni[:, None, :] * np.cross(nrm[:, None, :], c)


def tet_gradient(v, t, f):
    """diffgeo.py:880-920 (1-D or 2-D f)."""
    f = np.asarray(f)
    p0, p1, p2, p3 = (v[t[:, k]] for k in range(4))
    e0, e2, e3, e4, e5 = p1 - p0, p0 - p2, p3 - p0, p3 - p1, p3 - p2
    vol = np.abs(np.sum(e3 * np.cross(e0, e2), axis=1))
    vol[vol < EPS] = 1
    voli = np.divide(1.0, vol)[:, None]
    cr25, cr34, cr2e0 = np.cross(e2, e5), np.cross(e3, e4), np.cross(-e2, e0)
    if f.ndim == 1:
        d = [f[t[:, k], None] - f[t[:, 0], None] for k in (1, 2, 3)]
        return voli * (d[0] * cr25 + d[1] * cr34 + d[2] * cr2e0)
    d = [(f[t[:, k]] - f[t[:, 0]])[:, :, None] for k in (1, 2, 3)]
    return voli[:, None, :] * (d[0] * cr25[:, None, :] + d[1] * cr34[:, None, :] + d[2] * cr2e0[:, None, :])


def tria_divergence(v, t, g):
    """diffgeo.py:334-387, the vertex sums done with np.add.at."""
    g = np.asarray(g)
    p0, p1, p2 = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    e2, e0, e1 = p1 - p0, p2 - p1, p0 - p2
    nrm = np.cross(e2, -e1)
    ln = np.sqrt(np.sum(nrm * nrm, axis=1))
    ln[ln < EPS] = 1
    cots = [(e2 * (-e1)).sum(1) / ln, (e0 * (-e2)).sum(1) / ln, (e1 * (-e0)).sum(1) / ln]
    c0, c1, c2 = cots[0][:, None] * e0, cots[1][:, None] * e1, cots[2][:, None] * e2
    G = g if g.ndim == 3 else g[:, None, :]
    xs = [((c2 - c1)[:, None, :] * G).sum(-1), ((c0 - c2)[:, None, :] * G).sum(-1), ((c1 - c0)[:, None, :] * G).sum(-1)]
    out = np.zeros((v.shape[0], G.shape[1]))
    for k in range(3):
        np.add.at(out, t[:, k], xs[k])
    out = 0.5 * out
    return out[:, 0] if g.ndim == 2 else out


def tet_divergence(v, t, g):
    """diffgeo.py:953-1006, the vertex sums done with np.add.at."""
    g = np.asarray(g)
    p0, p1, p2, p3 = (v[t[:, k]] for k in range(4))
    e0, e1, e2, e3, e4 = p1 - p0, p2 - p1, p2 - p0, p3 - p0, p3 - p1
    ns = [np.cross(e1, e4), np.cross(e3, e2), np.cross(e0, e3), np.cross(e2, e0)]
    G = g if g.ndim == 3 else g[:, None, :]
    out = np.zeros((v.shape[0], G.shape[1]))
    for k in range(4):
        np.add.at(out, t[:, k], (ns[k][:, None, :] * G).sum(-1))
    out = -(1.0 / 6.0) * out
    return out[:, 0] if g.ndim == 2 else out


def normalize_rows(g, scaled=True):
    """g / ||g|| with nan_to_num (diffgeo.py:153-154); ``scaled`` divides by the
    largest component first so that tiny gradients do not underflow."""
    g = np.asarray(g, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        if scaled:
            s = np.max(np.abs(g), axis=-1, keepdims=True)
            q = g / s
            out = q / np.sqrt((q ** 2).sum(-1))[..., None]
        else:
            out = g / np.sqrt((g ** 2).sum(-1))[..., None]
    return np.nan_to_num(out)


def poisson_neumann_consistent(A, b):
    """Solution of the singular Neumann system A x = b on a connected mesh:
    the part of b along the constants is removed (making it consistent), one
    vertex is pinned to 0 and the reduced SPD system is solved by splu.  The
    reference instead factors the singular A (solver.py:873-877), whose result
    carries the inconsistent part of b amplified by the near-zero pivot."""
    b = np.asarray(b, dtype=np.float64)
    b = b - b.mean(axis=0)
    mask = np.ones(A.shape[0], dtype=bool)
    mask[0] = False
    Af = sparse.csc_matrix(A)[:, mask].tocsr()[mask, :].tocsc()
    x = np.zeros_like(b)
    x[mask] = splu(Af).solve(b[mask])
    return x


def geodesic_f(v, t, u, scaled=True, consistent=False):
    """compute_geodesic_f (diffgeo.py:144-165): gradient, normalise, divergence,
    Poisson with the identity mass, minus the minimum.  ``consistent`` solves
    the singular Poisson problem with poisson_neumann_consistent."""
    npe = t.shape[1]
    grad = tria_gradient(v, t, u) if npe == 3 else tet_gradient(v, t, u)
    gn = normalize_rows(grad, scaled)
    div = tria_divergence(v, t, gn) if npe == 3 else tet_divergence(v, t, gn)
    A, _ = assemble_scipy(v, t, lump=True)
    if consistent:
        x = poisson_neumann_consistent(A, div)
    else:
        x = poisson(A, sparse.eye(A.shape[0]), div)
    return x - x.min(axis=0)


def _normalize_tria(v, t):
    """Centroid (area-weighted triangle centres) to the origin, unit area
    (tria_mesh.py:990-1015, 1390-1405)."""
    p0, p1, p2 = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    cr = np.cross(p2 - p1, p0 - p2)
    areas = 0.5 * np.sqrt(np.sum(cr * cr, axis=1))
    total = areas.sum()
    c = np.sum(((p0 + p1 + p2) / 3.0) * (areas / total)[:, None], axis=0)
    return (1.0 / np.sqrt(total)) * (v - c)


def mean_curvature_flow(v, t, max_iter=30, stop_eps=1e-13, step=1.0):
    """tria_mean_curvature_flow (diffgeo.py:523-606): fixed stiffness of the
    normalised mesh, lumped mass of the current mesh, (M + step A) V = M V by
    a sparse LU, re-normalise, stop on sum_k (dv_k' M dv_k)^2 < stop_eps."""
    from scipy.sparse.linalg import spsolve

    v = _normalize_tria(np.asarray(v), t)
    A, _ = assemble_scipy(v, t, lump=True)
    for _ in range(max_iter):
        v_last = v
        _, M = assemble_scipy(v, t, lump=True)
        v = spsolve(sparse.csc_matrix(M + step * A), M @ v)
        v = _normalize_tria(v, t)
        dv = v - v_last
        if np.trace(np.square(dv.T @ (M @ dv))) < stop_eps:
            break
    return v


__all__ = ["tria_local", "tet_local", "assemble_scipy", "assemble_sorted", "csr_sorted_sum", "avg_edge_length",
           "eigs", "eigs_dense", "poisson", "diffusion", "tria_gradient", "tet_gradient", "tria_divergence", "tet_divergence",
           "normalize_rows", "geodesic_f", "poisson_neumann_consistent", "mean_curvature_flow", "TRIA_IJ", "TET_IJ"]
