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
import re
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _static_bytes() -> int:
    """LAPY_STATIC_SCRATCH_BYTES as the public header defines it."""
    hdr = (Path(__file__).resolve().parent.parent / "include" / "lapy_gb300.h").read_text()
    m = re.search(r"#define\s+LAPY_STATIC_SCRATCH_BYTES\s+\(\(size_t\)(\d+)\s*<<\s*(\d+)\)", hdr)
    assert m, "LAPY_STATIC_SCRATCH_BYTES not found in include/lapy_gb300.h"
    return int(m.group(1)) << int(m.group(2))


STATIC_BYTES = _static_bytes()


def _heat_system(level: int = 3, ncol: int = 3):
    """K = M + t A of a deformed icosphere (lumped mass) and ncol right-hand
    sides, on the device."""
    import torch

    from lapy_gb300 import Solver, meshes

    mesh = meshes.sh_deform(meshes.icosphere(level), seed=17)
    fem = Solver(mesh, lump=True)
    A = fem._A.as_f64()
    t = mesh.avg_edge_length() ** 2
    kv = fem._M.as_f64().on_pattern(A.indptr, A.indices, A.data.numel())
    kv.add_(A.data.double(), alpha=t)
    n = A.n
    rng = np.random.default_rng(5)
    B = torch.from_numpy(rng.standard_normal((n, ncol))).to("cuda")
    return A, kv, B


def _solve(L, A, kv, B, static: bool, mixed: int = 1):
    import torch

    from lapy_gb300 import _device, _lib

    n, ncol = B.shape
    seg = np.array([0, n], dtype=np.int32)
    X = torch.full_like(B, float("nan"))
    status = np.zeros(ncol, dtype=np.int32)
    relres = np.zeros(ncol, dtype=np.float64)
    iters = C.c_int64(0)
    args = (n, _device.dptr(A.indptr), _device.dptr(A.indices), _device.dptr(kv), kv.numel(), 1, seg.ctypes.data,
            ncol, _device.dptr(B), _device.dptr(X), 1e-10, 20000, mixed, 1e-4, status.ctypes.data,
            relres.ctypes.data, C.byref(iters))
    if static:
        st = L.lapy_pcg_solve_static(*args, _device.stream())
    else:
        ws = _device.workspace(L.lapy_pcg_solve_workspace_bytes(n, kv.numel(), 1, seg.ctypes.data, ncol, mixed))
        st = L.lapy_pcg_solve(*args, _device.dptr(ws), ws.numel(), _device.stream())
    _lib.check(st, "pcg_solve_static" if static else "pcg_solve")
    torch.cuda.synchronize()
    assert np.all(status == 0), status
    assert np.all(relres <= 1e-10), relres
    return X.cpu().numpy()


@pytest.mark.parametrize("mixed", [1, 0])
@pytest.mark.parametrize("ncol", [3, 20])
def test_static_scratch_solve_matches_workspace_solve(cuda_ok, mixed, ncol):
    """FP32-in-FP64 and FP64 solves, one and two column chunks (16 columns per chunk)."""
    from lapy_gb300 import _lib

    L = _lib.lib()
    A, kv, B = _heat_system(ncol=ncol)
    ref = _solve(L, A, kv, B, static=False, mixed=mixed)
    for _ in range(2):  # the array keeps the previous call's contents
        got = _solve(L, A, kv, B, static=True, mixed=mixed)
        np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-12 * np.abs(ref).max())


def _grid_heat_system(cells: int, ncol: int):
    """K = M + t A of the unit square split into cells x cells x 2 triangles."""
    import torch

    from lapy_gb300 import Solver, meshes

    mesh = meshes.square_grid(cells)
    fem = Solver(mesh, lump=True)
    A = fem._A.as_f64()
    kv = fem._M.as_f64().on_pattern(A.indptr, A.indices, A.data.numel())
    kv.add_(A.data.double(), alpha=mesh.avg_edge_length() ** 2)
    rng = np.random.default_rng(7)
    B = torch.from_numpy(rng.standard_normal((A.n, ncol))).to("cuda")
    return A, kv, B


def test_static_scratch_at_the_size_limit(cuda_ok):
    """The largest square grid (16 columns, one full chunk) whose scratch still
    fits the static array: solved twice, equal to the workspace solve."""
    from lapy_gb300 import _lib

    L = _lib.lib()

    def need(cells):  # (cells+1)^2 rows, 7 cells^2 + 6 cells + 1 nonzeros
        n = (cells + 1) ** 2
        seg = np.array([0, n], dtype=np.int32)
        return L.lapy_pcg_solve_workspace_bytes(n, 7 * cells * cells + 6 * cells + 1, 1, seg.ctypes.data, 16, 1)

    lo, hi = 8, 2048
    assert need(lo) <= STATIC_BYTES < need(hi)
    while hi - lo > 1:
        mid = (lo + hi) // 2
        lo, hi = (mid, hi) if need(mid) <= STATIC_BYTES else (lo, mid)
    assert need(lo) > 0.97 * STATIC_BYTES
    A, kv, B = _grid_heat_system(lo, 16)
    seg = np.array([0, A.n], dtype=np.int32)
    assert L.lapy_pcg_solve_workspace_bytes(A.n, kv.numel(), 1, seg.ctypes.data, 16, 1) == need(lo)
    ref = _solve(L, A, kv, B, static=False)
    for _ in range(2):
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
