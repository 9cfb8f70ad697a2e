"""Standalone FP32 SELL product (the inner PCG's SpMM outside the persistent
kernel) against SciPy's CSR product of the same matrix (GPU).

The reference multiplies by the stiffness matrix inside ARPACK's operator
(lapy/solver.py:707-713, ``splu(...).solve`` on ``A - sigma M``); this is the
product the FP32 inner iterations use.  Values are cast to FP32, so the bar is
FP32 accuracy against the FP64 product: |Y - A X| <= 1e-5 (|A| |X|)."""

from __future__ import annotations

import numpy as np
import pytest
from scipy import sparse

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ncol", [1, 2, 4, 8])
def test_sell_f32_spmm_matches_csr(cuda_ok, ncol):
    import torch

    from lapy_gb300 import _device, meshes, shapedna

    ms = meshes.deformed_icospheres([3, 5, 4, 3], [11, 12, 13, 14])
    fem = shapedna.BatchedFEM(ms, lump=False)
    sell = _device.SellF32(fem.indptr, fem.indices, fem.a_vals, fem.n, fem.nnz, seg_row=fem.seg_row)
    rng = np.random.default_rng(ncol)
    x = rng.standard_normal((fem.n, ncol)).astype(np.float32)
    y = torch.full((fem.n, ncol), float("nan"), device="cuda", dtype=torch.float32)
    sell.spmm(torch.from_numpy(x).cuda(), y)
    A = sparse.csr_matrix((fem.a_vals.cpu().numpy(), fem.indices.cpu().numpy(), fem.indptr.cpu().numpy()),
                          shape=(fem.n, fem.n))
    ref = A @ x.astype(np.float64)
    bound = abs(A) @ np.abs(x.astype(np.float64))
    got = y.cpu().numpy().astype(np.float64)
    assert np.all(np.isfinite(got))
    assert np.all(np.abs(got - ref) <= 1e-5 * bound + 1e-30)


def test_sell_f32_rejects_bad_width(cuda_ok):
    import torch

    from lapy_gb300 import _device, meshes, shapedna

    fem = shapedna.BatchedFEM(meshes.deformed_icospheres([3], [5]), lump=False)
    sell = _device.SellF32(fem.indptr, fem.indices, fem.a_vals, fem.n, fem.nnz, seg_row=fem.seg_row)
    x = torch.zeros(fem.n, 3, device="cuda", dtype=torch.float32)
    with pytest.raises(ValueError, match="ncol"):
        sell.spmm(x, torch.empty_like(x))
