"""IC(0) on the GPU against the restatement in oracle/ic0.py.

The factor is computed in the oracle's order without fused multiply-add, so
its entries must agree bit for bit; the triangular solves to rel 1e-12; the
preconditioned solve to the path's bar (FP64 true residual <= 1e-8, heat
M-norm rel <= 1e-8 against the reference's splu solve)."""

from __future__ import annotations

import numpy as np
import pytest
from scipy import sparse

import oracle
from oracle import ic0 as O

pytestmark = pytest.mark.gpu


def _systems():
    from lapy_gb300 import meshes

    out = []
    m = meshes.sh_deform(meshes.icosphere(3), seed=3)
    A, M = oracle.assemble_scipy(m.v, m.t)
    out.append(("shift", sparse.csr_matrix(A + 0.01 * M)))
    out.append(("heat", sparse.csr_matrix(M + 1e-3 * A)))
    k = meshes.kuhn_cube(5, jitter=0.2, seed=1)
    A, M = oracle.assemble_scipy(k.v, k.t)
    out.append(("tet", sparse.csr_matrix(A + 0.01 * M)))
    return out


def _dev(K):
    import torch

    K = sparse.csr_matrix(K)
    K.sort_indices()
    ip = torch.from_numpy(K.indptr.astype(np.int32)).cuda()
    ix = torch.from_numpy(K.indices.astype(np.int32)).cuda()
    kv = torch.from_numpy(K.data.astype(np.float64)).cuda()
    return ip, ix, kv


@pytest.mark.parametrize("case", range(3))
def test_ic0_factor_matches_oracle_bitwise(cuda_ok, case):
    from lapy_gb300 import _device

    name, K = _systems()[case]
    ip, ix, kv = _dev(K)
    lv, _, fixed, levels = _device.ic0_factor(ip, ix, kv, K.shape[0], K.nnz)
    Lref, fixed_ref = O.ic0(K)
    assert fixed == fixed_ref
    assert levels[0] == O.levels(K).max() + 1
    got = sparse.csr_matrix((lv.cpu().numpy(), K.indices, K.indptr), shape=K.shape)
    np.testing.assert_array_equal(sparse.tril(got).toarray(), Lref.toarray())
    np.testing.assert_array_equal(sparse.triu(got, 1).toarray(), sparse.triu(Lref.T, 1).toarray())


@pytest.mark.parametrize("case", range(3))
def test_ic0_apply_matches_oracle(cuda_ok, case):
    import torch

    from lapy_gb300 import _device

    _, K = _systems()[case]
    ip, ix, kv = _dev(K)
    lv, work, _, _ = _device.ic0_factor(ip, ix, kv, K.shape[0], K.nnz)
    Lref, _ = O.ic0(K)
    r = np.random.default_rng(1).standard_normal((K.shape[0], 3))
    z = _device.ic0_apply(ip, ix, lv, K.shape[0], K.nnz, torch.from_numpy(r).cuda(), work).cpu().numpy()
    zref = np.column_stack([O.ic0_apply(Lref, r[:, c]) for c in range(3)])
    np.testing.assert_allclose(z, zref, rtol=1e-12, atol=1e-12 * np.abs(zref).max())


@pytest.mark.parametrize("case", range(3))
def test_ic0_pcg_solves_to_tolerance_in_fewer_iterations(cuda_ok, case):
    import torch

    from lapy_gb300 import _device

    _, K = _systems()[case]
    ip, ix, kv = _dev(K)
    b = np.random.default_rng(2).standard_normal(K.shape[0])
    B = torch.from_numpy(b).cuda()
    x, relres, it_ic0, fixed = _device.ic0_pcg_solve(ip, ix, kv, K.shape[0], K.nnz, B, 1e-10)
    _, _, it_jac = _device.pcg_solve(ip, ix, kv, K.shape[0], K.nnz, B, 1e-10)
    x = x.cpu().numpy()
    assert np.linalg.norm(b - K @ x) <= 1e-8 * np.linalg.norm(b)
    assert fixed == 0
    assert it_ic0 < it_jac


def test_ic0_batched_heat_matches_reference(cuda_ok):
    from lapy_gb300 import heat, meshes

    ms = [meshes.sh_deform(meshes.icosphere(lv), seed=s) for lv, s in ((3, 1), (2, 2), (4, 3))]
    hb = heat.HeatBatch(ms, vids=0, m=1.0)
    x, info = hb.solve(precond="ic0")
    x = x.cpu().numpy()
    seg = hb.input.seg_row
    for i, m in enumerate(ms):
        ref = oracle.diffusion(m.v, m.t, 0, m=1.0)
        _, Ml = oracle.assemble_scipy(m.v, m.t, lump=True)
        w = Ml.diagonal()
        u = x[seg[i]:seg[i + 1]]
        assert np.sqrt(np.sum(w * (u - ref) ** 2) / np.sum(w * ref ** 2)) <= 1e-8
    u1 = heat.diffusion(ms[0], 0, m=1.0, precond="ic0")
    np.testing.assert_allclose(u1, oracle.diffusion(ms[0].v, ms[0].t, 0, m=1.0), rtol=1e-7,
                               atol=1e-9 * np.abs(u1).max())


def test_ic0_replaced_pivot_is_counted(cuda_ok):
    from lapy_gb300 import _device

    K = sparse.csr_matrix(np.array([[1.0, 2.0], [2.0, 1.0]]))
    ip, ix, kv = _dev(K)
    lv, _, fixed, _ = _device.ic0_factor(ip, ix, kv, 2, K.nnz)
    assert fixed == 1
    np.testing.assert_array_equal(lv.cpu().numpy(), [1.0, 2.0, 2.0, 1.0])
