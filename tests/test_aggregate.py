"""The aggregation and row order of the batched two-level eigensolver
(``lapy_aggregate_order``, host code, CPU): every segment's rows are
permuted within the segment, each aggregate is a contiguous, connected run of
rows numbered 0..nc-1 in order, sizes stay near the target, and repeated
calls (also after a larger problem) give the same result."""

from __future__ import annotations

import numpy as np
import pytest
from scipy import sparse
from scipy.sparse.csgraph import connected_components

import oracle
from lapy_gb300 import _lib, meshes


def _batch(levels, seeds):
    ms = meshes.deformed_icospheres(levels, seeds)
    A = sparse.block_diag([oracle.assemble_scipy(m.v, m.t)[0] for m in ms]).tocsr()
    A.sort_indices()
    seg = np.cumsum([0] + [len(m.v) for m in ms]).astype(np.int32)
    return A, seg


def _order(A, seg, target=64):
    L = _lib.lib()
    n = A.shape[0]
    ip = A.indptr.astype(np.int32)
    ix = A.indices.astype(np.int32)
    perm = np.full(n, -7, np.int32)
    lab = np.full(n, -7, np.int32)
    st = L.lapy_aggregate_order(n, ip.ctypes.data, ix.ctypes.data, seg.ctypes.data, len(seg) - 1, target,
                                perm.ctypes.data, lab.ctypes.data)
    assert st == 0, _lib.lib().lapy_last_error()
    return perm, lab


def test_aggregates_are_contiguous_connected_runs():
    A, seg = _batch([3, 4, 2, 3], [1, 2, 3, 4])
    perm, lab = _order(A, seg)
    for s in range(len(seg) - 1):
        r0, r1 = int(seg[s]), int(seg[s + 1])
        p = perm[r0:r1]
        assert np.array_equal(np.sort(p), np.arange(r0, r1))  # rows stay in their segment
        g = lab[r0:r1]
        if g[0] < 0:  # no coarse space for this segment: rows keep their order
            assert np.all(g == -1) and np.array_equal(p, np.arange(r0, r1))
            continue
        assert g[0] == 0 and np.all(np.diff(g) >= 0) and np.all(np.diff(g) <= 1)  # runs numbered in order
        nc = int(g[-1]) + 1
        sizes = np.bincount(g, minlength=nc)
        assert sizes.min() >= 1 and sizes.max() <= 3 * 64  # about the target, plus merged leftovers
        B = A[p][:, p].tocsr()
        for a in range(nc):
            rows = np.nonzero(g == a)[0]
            sub = B[rows][:, rows]
            assert connected_components(sub, directed=False)[0] == 1  # each aggregate is connected


def test_deterministic_and_independent_of_earlier_calls():
    A, seg = _batch([4, 3, 4], [7, 8, 9])
    first = _order(A, seg)
    big, bseg = _batch([5, 5], [10, 11])
    _order(big, bseg)  # a larger problem in between (scratch kept across calls)
    again = _order(A, seg)
    assert np.array_equal(first[0], again[0]) and np.array_equal(first[1], again[1])


def test_invalid_arguments_are_rejected():
    L = _lib.lib()
    A, seg = _batch([2], [1])
    n = A.shape[0]
    ip = A.indptr.astype(np.int32)
    ix = A.indices.astype(np.int32)
    perm = np.empty(n, np.int32)
    lab = np.empty(n, np.int32)
    bad = np.array([0, n - 1], np.int32)
    assert L.lapy_aggregate_order(n, ip.ctypes.data, ix.ctypes.data, bad.ctypes.data, 1, 64, perm.ctypes.data,
                                  lab.ctypes.data) == _lib.ERR_INVALID
    assert L.lapy_aggregate_order(n, ip.ctypes.data, ix.ctypes.data, seg.ctypes.data, 1, 32, perm.ctypes.data,
                                  lab.ctypes.data) == _lib.ERR_INVALID
