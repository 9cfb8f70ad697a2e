"""The allocation-free PCG entry point (lapy_pcg_solve_static) against the
workspace one (lapy_pcg_solve), through the C ABI.

lapy_pcg_solve_static serves callers that cannot allocate device memory: its
scratch is a static device array of LAPY_STATIC_SCRATCH_BYTES that the library
holds.  Two calls in a row must both reproduce the workspace solve, and a
problem larger than the array must be refused before any GPU work.  This file
is collected last so that a failure here leaves every other test already run.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATIC_BYTES = 32 << 20  # LAPY_STATIC_SCRATCH_BYTES in include/lapy_gb300.h


def _heat_system():
    """K = M + t A of a deformed icosphere (lumped mass) on the device."""
    import torch

    from lapy_gb300 import Solver, meshes

    mesh = meshes.sh_deform(meshes.icosphere(3), seed=17)
    fem = Solver(mesh, lump=True)
    A = fem._A.as_f64()
    t = mesh.avg_edge_length() ** 2
    kv = fem._M.as_f64().on_pattern(A.indptr, A.indices, A.data.numel())
    kv.add_(A.data.double(), alpha=t)
    n = A.n
    rng = np.random.default_rng(5)
    B = torch.from_numpy(rng.standard_normal((n, 3))).to("cuda")
    return A, kv, B


def _solve(L, A, kv, B, static: bool):
    import torch

    from lapy_gb300 import _device, _lib

    n, ncol = B.shape
    seg = np.array([0, n], dtype=np.int32)
    X = torch.full_like(B, float("nan"))
    status = np.zeros(ncol, dtype=np.int32)
    relres = np.zeros(ncol, dtype=np.float64)
    iters = C.c_int64(0)
    args = (n, _device.dptr(A.indptr), _device.dptr(A.indices), _device.dptr(kv), kv.numel(), 1, seg.ctypes.data,
            ncol, _device.dptr(B), _device.dptr(X), 1e-10, 20000, 1, 1e-4, status.ctypes.data, relres.ctypes.data,
            C.byref(iters))
    if static:
        st = L.lapy_pcg_solve_static(*args, _device.stream())
    else:
        ws = _device.workspace(L.lapy_pcg_solve_workspace_bytes(n, kv.numel(), 1, seg.ctypes.data, ncol, 1))
        st = L.lapy_pcg_solve(*args, _device.dptr(ws), ws.numel(), _device.stream())
    _lib.check(st, "pcg_solve_static" if static else "pcg_solve")
    torch.cuda.synchronize()
    assert np.all(status == 0), status
    assert np.all(relres <= 1e-10), relres
    return X.cpu().numpy()


def test_static_scratch_solve_matches_workspace_solve(cuda_ok):
    from lapy_gb300 import _lib

    L = _lib.lib()
    A, kv, B = _heat_system()
    ref = _solve(L, A, kv, B, static=False)
    for _ in range(2):  # the array keeps the previous call's contents
        got = _solve(L, A, kv, B, static=True)
        np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-12 * np.abs(ref).max())


def test_static_scratch_refuses_oversized_problem(cuda_ok):
    import torch

    from lapy_gb300 import _device, _lib

    L = _lib.lib()
    n, ncol = 2_000_000, 16
    seg = np.array([0, n], dtype=np.int32)
    need = L.lapy_pcg_solve_workspace_bytes(n, 7 * n, 1, seg.ctypes.data, ncol, 1)
    assert need > STATIC_BYTES
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")  # never read: the size check comes first
    status = np.zeros(ncol, dtype=np.int32)
    relres = np.zeros(ncol, dtype=np.float64)
    iters = C.c_int64(0)
    st = L.lapy_pcg_solve_static(n, _device.dptr(dummy), _device.dptr(dummy), _device.dptr(dummy), 7 * n, 1,
                                 seg.ctypes.data, ncol, _device.dptr(dummy), _device.dptr(dummy), 1e-10, 100, 1,
                                 1e-4, status.ctypes.data, relres.ctypes.data, C.byref(iters), _device.stream())
    assert st == _lib.ERR_WORKSPACE
    assert b"LAPY_STATIC_SCRATCH_BYTES" in L.lapy_last_error()
