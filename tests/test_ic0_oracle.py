"""The IC(0) restatement in oracle/ic0.py (CPU).

IC(0) has no counterpart in the reference (it factors exactly with SuperLU,
lapy/solver.py:707-712, lapy/heat.py:226); the restatement is checked by the
defining property of IC(0) - (L L')_ij = K_ij on the pattern of K - by its
effect as a preconditioner, and by the level structure the GPU schedules."""

from __future__ import annotations

import numpy as np
from scipy import sparse

import oracle
from oracle import ic0 as O


def _shift_system(level=3, seed=3):
    from lapy_gb300 import meshes

    m = meshes.sh_deform(meshes.icosphere(level), seed=seed)
    A, M = oracle.assemble_scipy(m.v, m.t)
    return sparse.csr_matrix(A + 0.01 * M), sparse.csr_matrix(M + 1e-3 * A)


def test_ic0_reproduces_k_on_its_pattern():
    for K in _shift_system():
        L, fixed = O.ic0(K)
        assert fixed == 0
        assert sparse.tril(L, -1).nnz + L.shape[0] == sparse.tril(K).nnz  # L on the lower pattern of K
        LL = (L @ L.T).tocsr()
        C = K.tocoo()
        err = np.abs(np.asarray(LL[C.row, C.col]).ravel() - C.data).max() / np.abs(C.data).max()
        assert err < 1e-14


def test_ic0_preconditions_better_than_jacobi():
    K, _ = _shift_system()
    L, _ = O.ic0(K)
    b = np.random.default_rng(0).standard_normal(K.shape[0])
    x, it_ic0 = O.pcg(K, b, lambda r: O.ic0_apply(L, r))
    _, it_jac = O.pcg(K, b, lambda r: r / K.diagonal())
    assert np.linalg.norm(b - K @ x) <= 1e-8 * np.linalg.norm(b)
    assert it_ic0 < 0.6 * it_jac


def test_icosphere_order_has_few_levels():
    from lapy_gb300 import meshes

    for level in (2, 4, 5):
        m = meshes.icosphere(level)
        A, _ = oracle.assemble_scipy(m.v, m.t)
        assert O.levels(A).max() + 1 <= 8


def test_nonpositive_pivot_is_replaced_and_counted():
    K = sparse.csr_matrix(np.array([[1.0, 2.0], [2.0, 1.0]]))
    L, fixed = O.ic0(K)
    assert fixed == 1
    np.testing.assert_array_equal(L.toarray(), [[1.0, 0.0], [2.0, 1.0]])
