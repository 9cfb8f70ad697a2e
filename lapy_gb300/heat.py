"""GPU drop-in for ``lapy.heat`` (lapy/heat.py).

``diffusion`` (heat.py:114-232): one backward-Euler step ``(M + t A) u = M
u0`` with lumped ``M`` and ``t = m * avg_edge_length**2``, for one or several
seed sets; the system is solved by FP32 Jacobi-PCG inside FP64 iterative
refinement instead of a sparse LU factorisation.  ``diagonal`` and ``kernel``
(heat.py:19-111): heat-kernel values from eigenpairs, the product over the
mesh's rows by a CUDA kernel.
"""

from __future__ import annotations

import logging

import numpy as np
import torch

from . import _lib
from ._device import axpby, dptr, ic0_pcg_solve, pcg_solve, require_cuda, stream

logger = logging.getLogger(__name__)


def _heat_product(evecs, sel, n: int, S, squared: bool) -> np.ndarray:
    """``np.matmul(W, S)`` for W = evecs[sel, 0:n] (squared element-wise when
    ``squared``), computed by the GPU product kernel.  ``sel`` holds row
    indices (any shape); S is the 1-D or 2-D factor the reference forms on the
    host.  Shapes follow np.matmul, and so do its errors (checked on empty
    stand-ins before any transfer)."""
    S = np.asarray(S, dtype=np.float64)
    w_shape = sel.shape + (n,)
    # numpy's own shape check on zero-strided stand-ins (no data, no product)
    stand_w = np.lib.stride_tricks.as_strided(np.zeros(1), shape=(1, n) if len(w_shape) > 1 else (n,),
                                              strides=(0, 0) if len(w_shape) > 1 else (0,))
    np.matmul(stand_w, np.zeros(S.shape))
    if S.ndim not in (1, 2):
        raise ValueError("the exp(-lambda t) factor must be 1-D or 2-D")
    out_shape = sel.shape + (S.shape[1],) if S.ndim == 2 else sel.shape
    nt = S.shape[1] if S.ndim == 2 else 1
    require_cuda()
    ev = np.asarray(evecs, dtype=np.float64)
    ev_d = torch.from_numpy(np.ascontiguousarray(ev)).to("cuda")
    rows = torch.from_numpy(np.ascontiguousarray(sel.reshape(-1), dtype=np.int64)).to("cuda")
    s_d = torch.from_numpy(np.ascontiguousarray(S.reshape(n, nt))).to("cuda")
    h = torch.empty((rows.numel(), nt), dtype=torch.float64, device="cuda")
    _lib.check(_lib.lib().lapy_heat_product_f64(rows.numel(), dptr(rows), dptr(ev_d), ev.shape[1], n, int(squared),
                                                 dptr(s_d), nt, dptr(h), stream()), "heat_product")
    res = h.cpu().numpy().reshape(out_shape)
    return res[()] if res.ndim == 0 else res


def diagonal(t, x, evecs, evals, n: int) -> np.ndarray:
    """Heat kernel diagonal K(t, x, x) from the first n eigenpairs
    (lapy/heat.py:19-60): ``evecs[x, :n]**2 @ exp(-evals[:n] @ t)``.  The
    exponent matrix is formed on the host exactly as the reference does (so
    ``evals`` as a column and ``t`` as a row give one column per time); the
    product over the mesh's rows runs on the GPU."""
    evecs = np.asarray(evecs)
    evals = np.asarray(evals)
    if n > evecs.shape[1] or n > evals.shape[0]:
        raise ValueError("n exceeds the number of available eigenpairs")
    S = np.exp(-np.matmul(evals[0:n], t))
    sel = np.arange(evecs.shape[0])[x]
    return _heat_product(evecs, np.asarray(sel), n, S, squared=True)


def kernel(t, vfix: int, evecs, evals, n: int) -> np.ndarray:
    """Heat kernel K_t(p, vfix) for all p from the first n eigenpairs
    (lapy/heat.py:63-111): ``evecs[:, :n] @ (exp(-evals[:n] @ t) *
    evecs[vfix, :n])``, the factor formed on the host with the reference's
    broadcasting, the product on the GPU."""
    evecs = np.asarray(evecs)
    evals = np.asarray(evals)
    if n > evecs.shape[1] or n > evals.shape[0]:
        raise ValueError("n exceeds the number of available eigenpairs")
    S = np.exp(np.matmul(-evals[0:n], t)) * evecs[vfix, 0:n]
    return _heat_product(evecs, np.arange(evecs.shape[0]), n, S, squared=False)


def diffusion(geometry, vids, m: float = 1.0, aniso=None, use_cholmod: bool = False, rtol: float = 1e-11,
              precond: str = "jacobi"):
    """Heat diffusion from the vertices in ``vids`` (same semantics as the reference).

    ``precond``: ``"jacobi"``, ``"ic0"`` (incomplete Cholesky) or ``"learned"``
    (the shipped per-edge MLP sparse approximate inverse; isotropic systems
    only)."""
    if precond not in ("jacobi", "ic0", "learned"):
        raise ValueError(f"precond must be 'jacobi', 'ic0' or 'learned', not {precond!r}")
    if precond == "learned" and aniso is not None:
        raise ValueError("the learned preconditioner covers isotropic systems (aniso=None)")
    if use_cholmod:
        from .solver import _import_optional

        _import_optional("sksparse")
    from .solver import Solver

    nv = len(geometry.v)
    if isinstance(vids, list) and len(vids) > 0 and isinstance(vids[0], (list, np.ndarray)):
        scalar_input = False
        vids_list = [np.asarray(v, dtype=int).ravel() for v in vids]
    else:
        scalar_input = True
        vids_list = [np.asarray(vids, dtype=int).ravel()]
    for v in vids_list:
        if np.any(v < 0) or np.any(v >= nv):
            raise ValueError("vids contains out-of-range vertex indices")

    fem = Solver(geometry, lump=True, aniso=aniso)
    t = m * geometry.avg_edge_length() ** 2
    A = fem._A.as_f64()
    n = A.n
    # hmat = M + t A on A's pattern (lumped M added to the diagonal)
    L = _lib.lib()
    hvals = fem._M.as_f64().on_pattern(A.indptr, A.indices, A.data.numel())
    axpby(t, A.data.double().contiguous(), 1.0, hvals, out=hvals)
    n_cases = len(vids_list)
    b0 = np.zeros((nv, n_cases))
    for k, v in enumerate(vids_list):
        b0[v, k] = 1.0
    if n != nv:
        raise ValueError(f"mesh has {nv} vertices but its elements reference only {n}")
    B = torch.from_numpy(b0).to("cuda")
    if precond == "learned":
        from .shapedna import BatchInput
        from .spai import SpaiSystems, learned_solve

        sysg = SpaiSystems(BatchInput([geometry]), "heat", t=[t])
        x, relres, iters = learned_solve(sysg, B, rtol)
    elif precond == "ic0":
        x, relres, iters, _ = ic0_pcg_solve(A.indptr, A.indices, hvals, n, hvals.numel(), B, rtol)
    else:
        x, relres, iters = pcg_solve(A.indptr, A.indices, hvals, n, hvals.numel(), B, rtol)
    logger.debug("heat solve: %d PCG iterations, max rel. residual %.2e", iters, float(np.max(relres)))
    vfunc = x.cpu().numpy()
    del L
    if scalar_input:
        return vfunc[:, 0]
    return vfunc


class HeatBatch:
    """Backward-Euler heat systems of a batch of meshes on the device.

    Each mesh s of the block-diagonal batch gets its own
    ``t_s = m * avg_edge_length_s**2`` (lapy/heat.py:206) and the system
    ``(M_s + t_s A_s) u = b0_s`` with lumped ``M`` (lapy/heat.py:204, 208); all
    segments are solved by one batched PCG launch sequence."""

    def __init__(self, batch_input, vids=0, m: float = 1.0):
        from .shapedna import BatchInput

        if not isinstance(batch_input, BatchInput):
            batch_input = BatchInput(batch_input)
        self.input = batch_input
        self.m = float(m)
        seg = batch_input.seg_row
        nseg = len(seg) - 1
        sizes = np.diff(seg)
        v = np.asarray(vids, dtype=np.int64).reshape(-1)
        if v.size == 1:
            v = np.full(nseg, v[0])
        if len(v) != nseg:
            raise ValueError("vids needs one vertex per mesh (or one vertex for all)")
        if np.any(v < 0) or np.any(v >= sizes):
            raise ValueError("vids contains out-of-range vertex indices")
        vid = torch.from_numpy(v.astype(np.int32)).to("cuda")
        self.b0 = torch.empty(int(seg[-1]), dtype=torch.float64, device="cuda")
        _lib.check(_lib.lib().lapy_seg_unit_vector(int(seg[-1]), nseg, dptr(batch_input.seg_row_dev), dptr(vid),
                                                   dptr(self.b0), stream()), "seg_unit_vector")
        self.ones = torch.ones(nseg, dtype=torch.float64, device="cuda")

    def solve(self, rtol: float = 1e-11, maxiter: int = 20000, precond: str = "jacobi"):
        """Assemble and solve every segment; returns (u (n,), info).
        ``precond``: ``"jacobi"``, ``"ic0"`` or ``"learned"`` (per-edge MLP SPAI)."""
        from .shapedna import BatchedFEM

        inp = self.input
        fem = BatchedFEM.from_input(inp, lump=True)
        L = _lib.lib()
        nseg = len(inp.seg_row) - 1
        seg_dev = inp.seg_row_dev
        avg = torch.empty(nseg, dtype=torch.float64, device="cuda")
        t = torch.empty(nseg, dtype=torch.float64, device="cuda")
        _lib.check(L.lapy_seg_avg_edge_length(dptr(inp.mesh.v), inp.mesh.coords_f32, nseg, dptr(seg_dev),
                                              dptr(fem.indptr), dptr(fem.indices), self.m, dptr(avg), dptr(t),
                                              stream()), "seg_avg_edge_length")
        hvals = torch.empty(fem.nnz, dtype=torch.float64, device="cuda")
        _lib.check(L.lapy_csr_seg_axpby(nseg, dptr(seg_dev), dptr(fem.indptr), dptr(fem.pattern.diag_pos),
                                        dptr(t), dptr(fem.a_vals), dptr(self.ones), dptr(fem.m_vals), 1,
                                        dptr(hvals), stream()), "csr_seg_axpby")
        if precond == "learned":
            from .spai import SpaiSystems, learned_solve

            x, relres, iters = learned_solve(SpaiSystems(inp, "heat", t=t), self.b0, rtol, maxiter)
        elif precond == "jacobi":
            x, relres, iters = pcg_solve(fem.indptr, fem.indices, hvals, fem.n, fem.nnz, self.b0, rtol, maxiter,
                                         seg_row=inp.seg_row)
        elif precond == "ic0":
            x, relres, iters, _ = ic0_pcg_solve(fem.indptr, fem.indices, hvals, fem.n, fem.nnz, self.b0, rtol,
                                                maxiter, seg_row=inp.seg_row)
        else:
            raise ValueError(f"precond must be 'jacobi', 'ic0' or 'learned', not {precond!r}")
        return x, {"relres": relres, "iters": iters, "t": t, "avg_edge_length": avg}


def diffusion_batch(meshes, vids=0, m: float = 1.0, rtol: float = 1e-11, precond: str = "jacobi") -> list:
    """Heat diffusion on many meshes at once: ``diffusion(mesh_s, vids[s], m)``
    for every mesh, solved as one block-diagonal batch.  ``vids``: one vertex
    per mesh, or one vertex index used for all meshes."""
    hb = HeatBatch(meshes, vids, m)
    x, _ = hb.solve(rtol, precond=precond)
    u = x.cpu().numpy()
    seg = hb.input.seg_row
    return [u[seg[i]:seg[i + 1]] for i in range(len(seg) - 1)]
