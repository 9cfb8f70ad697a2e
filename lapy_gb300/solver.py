"""GPU drop-in for ``lapy.Solver`` (lapy/solver.py).

Same constructor, attributes and methods as the reference:

* ``Solver(geometry, lump=False, aniso=None, aniso_smooth=10, use_cholmod=False,
  dtype=np.float64)`` assembles the cotangent stiffness ``A`` and the mass
  ``M`` on the GPU (lapy/solver.py:54-103), into a deterministic CSR pattern;
* ``.stiffness`` / ``.mass`` are SciPy ``csc_matrix`` views materialised on
  first access (device CSR underneath); assigning a SciPy matrix uploads it
  (lapy/diffgeo.py:149 replaces the mass by the identity);
* ``.eigs(k, sigma)`` solves ``A x = lambda M x`` by block shift-invert
  Lanczos on the GPU (lapy/solver.py:667-716);
* ``.poisson(h, dtup, ntup)`` (lapy/solver.py:718-889) with FP32 PCG inside
  FP64 iterative refinement.

There is no CPU fallback; without a GPU the constructor raises.
"""

from __future__ import annotations

import ctypes as C
import importlib
import logging

import numpy as np
import torch
from scipy import sparse

from . import _lib
from ._device import (DeviceCSR, assemble, dptr, mesh_device, pattern_of, pcg_solve, require_cuda, stream,
                      tria_curvature, workspace)

logger = logging.getLogger(__name__)

#: block width of the Lanczos iteration: >= the largest eigenvalue multiplicity
#: expected (the icosahedral symmetry of icospheres gives groups of up to 5)
DEFAULT_BLOCK = 8


def _import_optional(name: str):
    try:
        return importlib.import_module(name)
    except ImportError as exc:  # same behaviour as lapy/utils/_imports.py:52-61
        raise ImportError(f"Missing optional dependency '{name}'. Use pip or conda to install {name}.") from exc


class Solver:
    """FEM solver for Laplace eigenvalue and Poisson problems on the GPU."""

    def __init__(self, geometry, lump: bool = False, aniso=None, aniso_smooth: int = 10,
                 use_cholmod: bool = False, dtype=np.float64) -> None:
        if use_cholmod:
            # the reference requires scikit-sparse here; the GPU path never uses CHOLMOD
            _import_optional("sksparse")
        dtype = np.dtype(dtype)
        gname = type(geometry).__name__
        aniso_inputs = None
        if gname == "TriaMesh":
            if aniso is not None:
                logger.info("TriaMesh with anisotropic Laplace-Beltrami")
                if isinstance(aniso, (list, tuple, set, np.ndarray)):
                    if len(aniso) != 2:
                        raise ValueError("aniso should be scalar or tuple/array of length 2!")
                    aniso0, aniso1 = list(aniso)
                else:
                    aniso0 = aniso1 = aniso
                # curvature frame on the device (lapy/tria_mesh.py:1221-1279);
                # the two curvature weights exp(-a |c|) (solver.py:88-90) are
                # formed on the host from the m pooled curvatures
                md, pat = pattern_of(geometry)
                _, tri = tria_curvature(md, pat, aniso_smooth, vertex=False, triangle=True)
                m = md.m
                c = tri[6 * m:].cpu().numpy()
                c1, c2 = c[:m], c[m:]
                aniso_mat = np.empty((m, 2), dtype=dtype)
                aniso_mat[:, 1] = np.exp(-aniso1 * np.abs(c1))
                aniso_mat[:, 0] = np.exp(-aniso0 * np.abs(c2))
                aniso_inputs = (tri[:3 * m].view(m, 3), tri[3 * m:6 * m].view(m, 3), aniso_mat)
            else:
                logger.info("TriaMesh with regular Laplace-Beltrami")
        elif gname == "TetMesh":
            logger.info("TetMesh with regular Laplace")
        else:
            raise ValueError('Geometry type "' + gname + '" unknown')
        require_cuda()
        md, pat = pattern_of(geometry)
        out_dtype = torch.float32 if dtype == np.float32 else torch.float64
        a, m = assemble(md, pat, lump, out_dtype, aniso_inputs)
        self._pattern = pat
        self._mesh_dev = md
        self._A = DeviceCSR(pat.n, pat.indptr, pat.indices, a)
        self._M = DeviceCSR(pat.n, diag=m) if lump else DeviceCSR(pat.n, pat.indptr, pat.indices, m)
        self._A_host = None
        self._M_host = None
        self.geotype = type(geometry)
        self.use_cholmod = use_cholmod
        self._dtype = dtype

    # -- matrices ------------------------------------------------------------
    @property
    def stiffness(self) -> sparse.csc_matrix:
        if self._A_host is None:
            self._A_host = self._A.to_scipy()
        return self._A_host

    @stiffness.setter
    def stiffness(self, mat) -> None:
        self._A = DeviceCSR.from_scipy(mat)
        self._A_host = mat

    @property
    def mass(self) -> sparse.csc_matrix:
        if self._M_host is None:
            self._M_host = self._M.to_scipy()
        return self._M_host

    @mass.setter
    def mass(self, mat) -> None:
        self._M = DeviceCSR.from_scipy(mat)
        self._M_host = mat

    @staticmethod
    def fem_tria_mass(tria, lump: bool = False, dtype=np.float64) -> sparse.csc_matrix:
        """Mass matrix only (lapy/solver.py:310-377): the reference's ``vol`` here
        is the area, so its entries equal those of the full assembly's mass
        (vol/24 with vol = 4 * area is area/6)."""
        require_cuda()
        md, pat = pattern_of(tria)
        out_dtype = torch.float32 if np.dtype(dtype) == np.float32 else torch.float64
        _, m = assemble(md, pat, lump, out_dtype)
        M = DeviceCSR(pat.n, diag=m) if lump else DeviceCSR(pat.n, pat.indptr, pat.indices, m)
        return M.to_scipy()

    # -- eigenproblem ----------------------------------------------------------
    def _device_pair(self):
        """A (CSR, f64) and M on A's pattern or as a diagonal."""
        A = self._A.as_f64()
        if A.is_diag:
            raise _lib.LapyGpuError(_lib.ERR_PATTERN, "Solver", "a diagonal stiffness matrix is not supported")
        M = self._M.as_f64()
        if M.is_diag:
            return A, M.diag.contiguous(), True
        if M.indptr is A.indptr and M.indices is A.indices:
            return A, M.data.contiguous(), False
        return A, M.on_pattern(A.indptr, A.indices, A.data.numel()), False

    def eigs(self, k: int = 10, sigma: float = -0.01, block: int | None = None, tol: float = 1e-8,
             inner_rtol: float = 1e-9, precond: str = "twolevel"):
        """The k eigenpairs of A x = lambda M x nearest ``sigma`` (ascending).

        ``precond`` selects the inner PCG's preconditioner: ``"twolevel"``
        (Jacobi plus an aggregation coarse space) or ``"jacobi"``."""
        A, mvals, m_diag = self._device_pair()
        n = A.n
        if not (0 < k < n):
            raise ValueError(f"k must satisfy 0 < k < n = {n}")
        block = block or DEFAULT_BLOCK
        while block > 1 and n < k + 2 * block + 1:
            block //= 2
        evals, evecs, info = eigs_batched(A.indptr, A.indices, A.data.contiguous(), mvals, m_diag,
                                          np.array([0, n], dtype=np.int32), k, sigma, block, tol, inner_rtol,
                                          precond=precond)
        st = int(info["status"][0])
        if st != 0:
            _lib.check(st, "Solver.eigs")
        self.last_eigs_info = info
        return evals[0].cpu().numpy(), evecs.cpu().numpy()

    # -- Poisson ---------------------------------------------------------------
    def _masked_solve(self, A: DeviceCSR, b: torch.Tensor, mask: np.ndarray, rtol: float) -> torch.Tensor:
        """Solve A x = b with the rows/columns of masked vertices replaced by
        identity rows (their entries of b zeroed): the reduced system
        A[free][:, free] of lapy/solver.py:848-865 without forming it."""
        L = _lib.lib()
        maskd = torch.from_numpy(mask).to("cuda")
        kv = torch.empty_like(A.data.double())
        _lib.check(L.lapy_csr_dirichlet_mask(A.n, dptr(A.indptr), dptr(A.indices), dptr(A.data.double().contiguous()),
                                             dptr(maskd), dptr(kv), stream()), "csr_dirichlet_mask")
        b = b.clone()
        b[maskd.bool()] = 0.0
        x, _, _ = pcg_solve(A.indptr, A.indices, kv, A.n, kv.numel(), b, rtol)
        return x

    def poisson(self, h=0.0, dtup=(), ntup=(), rtol: float = 1e-12):
        """Poisson equation A x = M (h - n) with Dirichlet/Neumann data (lapy/solver.py:718-889)."""
        dim = self._A.n
        dtype = np.dtype(self._dtype) if self._A_host is None else self.stiffness.dtype
        if self._M.n != dim:
            raise ValueError("Error: Square input matrices should have same number of rows and columns.")
        if np.isscalar(h):
            h = np.full((dim, 1), h, dtype=dtype)
        else:
            h = np.asarray(h, dtype=dtype)
            if h.ndim == 1:
                if h.size != dim:
                    raise ValueError("h should be either scalar or column vector with row num of A")
                h = h[:, np.newaxis]
            elif h.ndim == 2:
                if h.shape[0] != dim:
                    raise ValueError("h should be either scalar or array with first dim matching A")
            else:
                raise ValueError("h should be either scalar or 1-D/2-D array")
        n_rhs = h.shape[1]
        scalar_rhs = n_rhs == 1
        didx = np.array([], dtype=np.int64)
        ddense = None
        if dtup:
            if len(dtup) != 2:
                raise ValueError("dtup should contain index and data arrays")
            didx = np.asarray(dtup[0])
            ddat = np.asarray(dtup[1], dtype=np.float64)
            if np.unique(didx).size != len(didx):
                raise ValueError("dtup indices need to be unique")
            if not (len(didx) > 0 and len(didx) == len(ddat)):
                raise ValueError("dtup should contain index and data arrays (same lengths > 0)")
            ddense = np.zeros((dim, n_rhs))
            ddense[didx, :] = ddat[:, None]
        nvec = None
        if ntup:
            if len(ntup) != 2:
                raise ValueError("ntup should contain index and data arrays")
            nidx = np.asarray(ntup[0])
            ndat = np.asarray(ntup[1], dtype=np.float64)
            if not (len(nidx) > 0 and len(nidx) == len(ndat)):
                raise ValueError("ntup should contain index and data arrays (same lengths > 0)")
            nvec = np.zeros((dim, n_rhs))
            np.add.at(nvec, nidx, ndat[:, None])
        require_cuda()
        rhs = h.astype(np.float64) if nvec is None else h.astype(np.float64) - nvec
        Hd = torch.from_numpy(np.ascontiguousarray(rhs)).to("cuda")
        M = self._M.as_f64()
        A = self._A.as_f64()
        b = M.matmul(Hd)
        L = _lib.lib()
        if ddense is not None:
            Dd = torch.from_numpy(np.ascontiguousarray(ddense)).to("cuda")
            b = b - A.matmul(Dd)
            mask = np.zeros(dim, dtype=np.uint8)
            mask[didx] = 1
            x = self._masked_solve(A, b, mask, rtol)
            md = torch.from_numpy(mask).to("cuda").bool()
            x[md] = Dd[md]
        else:
            # Neumann everywhere: A is singular (constants span its kernel on a
            # connected mesh).  The reference's LU returns one solution with an
            # arbitrary constant.  Here b is made consistent (mean removed), one
            # vertex is pinned to 0, which leaves an SPD system with the same
            # solutions up to a constant, and the zero-mean solution is returned.
            b = b - b.mean(dim=0, keepdim=True)
            mask = np.zeros(dim, dtype=np.uint8)
            mask[0] = 1
            x = self._masked_solve(A, b, mask, rtol)
            x = x - x.mean(dim=0, keepdim=True)
        x = x.cpu().numpy().astype(dtype, copy=False)
        if scalar_rhs:
            return np.squeeze(np.array(x))
        return np.array(x)


def eigs_batched(indptr, indices, a_vals, m_vals, m_is_diag: bool, seg_row, k: int, sigma: float = -0.01,
                 block: int = DEFAULT_BLOCK, tol: float = 1e-8, inner_rtol: float = 1e-9, inner_maxiter: int = 20000,
                 max_vectors: int | None = None, seed: int = 1234, precond: str = "twolevel",
                 tuning: dict | None = None):
    """Shift-invert eigenpairs of every segment of a block-diagonal batch.

    ``tuning``: solver knobs (``agg_target``, ``round_rtol``, ``fold_pieces``,
    ``fold_aggs``, ``ctas_per_sm``; missing keys keep the defaults), e.g. the
    choice of ``lapy_gb300.autotune``.
    Returns (evals: nseg x k tensor, evecs: n x k tensor, info dict)."""
    L = _lib.lib()
    pc = {"jacobi": _lib.PRECOND_JACOBI, "twolevel": _lib.PRECOND_TWO_LEVEL}.get(precond)
    if pc is None:
        raise ValueError(f"precond must be 'jacobi' or 'twolevel', not {precond!r}")
    seg_row = np.ascontiguousarray(seg_row, dtype=np.int32)
    nseg = len(seg_row) - 1
    n = int(seg_row[-1])
    nnz = int(a_vals.numel())
    if max_vectors is None:
        max_vectors = 6 * k + 8 * block
    ws_bytes = L.lapy_eigs_workspace_bytes(n, nnz, nseg, seg_row.ctypes.data, k, block, max_vectors, pc)
    ws = workspace(ws_bytes)
    evals = torch.empty(nseg, k, dtype=torch.float64, device="cuda")
    evecs = torch.empty(n, k, dtype=torch.float64, device="cuda")
    status = np.zeros(nseg, dtype=np.int32)
    nbasis = np.zeros(nseg, dtype=np.int32)
    iters = C.c_int64(0)
    tn = _lib.EigsTuning()
    for key, val in (tuning or {}).items():
        if key not in ("agg_target", "round_rtol", "fold_pieces", "fold_aggs", "ctas_per_sm"):
            raise ValueError(f"unknown tuning key {key!r}")
        setattr(tn, key, val)
    _lib.check(L.lapy_eigs_shift_invert_tuned(n, dptr(indptr), dptr(indices), dptr(a_vals), dptr(m_vals),
                                              int(m_is_diag), nnz, nseg, seg_row.ctypes.data, sigma, k, block,
                                              max_vectors, tol, inner_rtol, inner_maxiter, pc, seed, dptr(evals),
                                              dptr(evecs), status.ctypes.data, nbasis.ctypes.data, C.byref(iters),
                                              dptr(ws), ws.numel(), stream(), C.byref(tn)), "eigs_shift_invert")
    info = {"status": status, "nbasis": nbasis, "inner_iters": int(iters.value), "block": block, "precond": precond,
            "workspace_bytes": int(ws_bytes), "tuning": dict(tuning or {})}
    return evals, evecs, info
