"""GPU drop-in for ``lapy.heat.diffusion`` (lapy/heat.py:114-232).

One backward-Euler step ``(M + t A) u = M u0`` with lumped ``M`` and
``t = m * avg_edge_length**2``, for one or several seed sets; the system is
solved by FP32 Jacobi-PCG inside FP64 iterative refinement instead of a sparse
LU factorisation.
"""

from __future__ import annotations

import logging

import numpy as np
import torch

from . import _lib
from ._device import pcg_solve

logger = logging.getLogger(__name__)


def diffusion(geometry, vids, m: float = 1.0, aniso=None, use_cholmod: bool = False, rtol: float = 1e-11):
    """Heat diffusion from the vertices in ``vids`` (same semantics as the reference)."""
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
    hvals.add_(A.data.double(), alpha=t)
    n_cases = len(vids_list)
    b0 = np.zeros((nv, n_cases))
    for k, v in enumerate(vids_list):
        b0[v, k] = 1.0
    if n != nv:
        raise ValueError(f"mesh has {nv} vertices but its elements reference only {n}")
    B = torch.from_numpy(b0).to("cuda")
    x, relres, iters = pcg_solve(A.indptr, A.indices, hvals, n, hvals.numel(), B, rtol)
    logger.debug("heat solve: %d PCG iterations, max rel. residual %.2e", iters, float(np.max(relres)))
    vfunc = x.cpu().numpy()
    del L
    if scalar_input:
        return vfunc[:, 0]
    return vfunc
