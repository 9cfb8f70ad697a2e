"""Incomplete Cholesky IC(0) restatement (test infrastructure only).

The reference has no incomplete factorization: its solves factor exactly with
SuperLU (lapy/solver.py:707-712 for the shift-invert operator, lapy/heat.py:226
for the heat step).  IC(0) is the classical fallback preconditioner for the
same SPD systems on the GPU; this module restates it from the textbook
algorithm (Meijerink and van der Vorst, 1977) so the CUDA factor and solves
can be checked entry by entry:

    for each row i, for each lower entry (i, j), j < i, in ascending j:
        L[i, j] = (K[i, j] - sum_{m < j} L[i, m] L[j, m]) / L[j, j]
    L[i, i] = sqrt(K[i, i] - sum_{m < i} L[i, m]^2)

with the sums over the columns m present in both rows' lower patterns, taken
in ascending m and accumulated left to right (the CUDA kernel uses the same
order and no fused multiply-add, so the factors agree to the last bit).  A
pivot that is not positive is replaced by K[i, i] (diagonal compensation) and
counted.  Pure Python loops: small systems only.
"""

from __future__ import annotations

import math

import numpy as np
from scipy import sparse


def ic0(K):
    """IC(0) of the SPD CSR matrix K (sorted indices, full diagonal).

    Returns (L as a CSR matrix on the lower pattern of K, number of
    compensated pivots)."""
    K = sparse.csr_matrix(K)
    K.sort_indices()
    n = K.shape[0]
    ip, ix, kv = K.indptr, K.indices, K.data
    lower = [[(int(ix[k]), float(kv[k])) for k in range(ip[i], ip[i + 1]) if ix[k] <= i] for i in range(n)]
    Lrows = []  # per row: dict col -> value (lower part incl. diagonal)
    fixed = 0
    for i in range(n):
        row = {}
        cols_i = []
        diag = None
        for j, kij in lower[i]:
            if j == i:
                diag = kij
                continue
            Lj = Lrows[j]
            acc = 0.0
            for m in cols_i:  # ascending, all < j
                if m in Lj:
                    acc = acc + row[m] * Lj[m]
            row[j] = (kij - acc) / Lj[j]
            cols_i.append(j)
        if diag is None:
            raise ValueError(f"row {i} has no diagonal entry")
        acc = 0.0
        for m in cols_i:
            acc = acc + row[m] * row[m]
        d = diag - acc
        if not (d > 0.0) or not math.isfinite(d):
            d = diag
            fixed += 1
        row[i] = math.sqrt(d)
        Lrows.append(row)
    rows, cols, vals = [], [], []
    for i, row in enumerate(Lrows):
        for j in sorted(row):
            rows.append(i)
            cols.append(j)
            vals.append(row[j])
    L = sparse.csr_matrix((vals, (rows, cols)), shape=(n, n))
    return L, fixed


def ic0_apply(L, r):
    """z = (L L')^{-1} r by a forward and a backward triangular solve."""
    from scipy.sparse.linalg import spsolve_triangular

    y = spsolve_triangular(sparse.csr_matrix(L), np.asarray(r, dtype=np.float64), lower=True)
    return spsolve_triangular(sparse.csr_matrix(L.T), y, lower=False)


def levels(K):
    """Forward level of every row: 0 for rows with no lower off-diagonal
    entry, else 1 + the largest level among their lower neighbours (the
    dependency depth of the forward solve and of the row-wise factorization)."""
    K = sparse.csr_matrix(K)
    n = K.shape[0]
    lv = np.zeros(n, dtype=np.int64)
    for i in range(n):
        js = K.indices[K.indptr[i]:K.indptr[i + 1]]
        js = js[js < i]
        lv[i] = lv[js].max() + 1 if js.size else 0
    return lv


def pcg(K, b, apply, rtol=1e-8, maxiter=10000):
    """Preconditioned CG in FP64 (returns x, iterations)."""
    x = np.zeros_like(b)
    r = b.copy()
    z = apply(r)
    p = z.copy()
    rz = r @ z
    bb = b @ b
    for it in range(maxiter):
        q = K @ p
        a = rz / (p @ q)
        x += a * p
        r -= a * q
        if r @ r <= rtol * rtol * bb:
            return x, it + 1
        z = apply(r)
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
    return x, maxiter


__all__ = ["ic0", "ic0_apply", "levels", "pcg"]
