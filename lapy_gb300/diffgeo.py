"""GPU drop-ins for the heat-method geodesic pieces of lapy/diffgeo.py.

``compute_gradient`` (diffgeo.py:26-54), ``compute_divergence`` (:57-85) and
``compute_geodesic_f`` (:116-165) for triangle and tetrahedral meshes, with
1-D or 2-D vertex functions.  The gradient, the normalisation and the
integrated divergence are CUDA kernels; the Poisson step is
``Solver.poisson`` with the identity mass, as in the reference.
"""

from __future__ import annotations

import numpy as np
import torch
from scipy import sparse

from . import _lib
from ._device import dptr, pattern_of, require_cuda, stream


def _kind(geom) -> int:
    name = type(geom).__name__
    if name == "TriaMesh":
        return 3
    if name == "TetMesh":
        return 4
    raise ValueError('Geometry type "' + name + '" not implemented')


def _gradient_dev(geom, f: torch.Tensor) -> torch.Tensor:
    L = _lib.lib()
    npe = _kind(geom)
    md, _ = pattern_of(geom)
    nf = f.shape[1]
    out = torch.empty(md.m, nf, 3, dtype=torch.float64, device="cuda")
    fn = L.lapy_tria_gradient if npe == 3 else L.lapy_tet_gradient
    _lib.check(fn(dptr(md.v), md.coords_f32, dptr(md.t), md.m, dptr(f), nf, dptr(out), stream()), "gradient")
    return out


def _divergence_dev(geom, g: torch.Tensor) -> torch.Tensor:
    L = _lib.lib()
    npe = _kind(geom)
    md, pat = pattern_of(geom)
    nf = g.shape[1]
    out = torch.empty(md.n, nf, dtype=torch.float64, device="cuda")
    work = torch.empty(md.m * npe * nf, dtype=torch.float64, device="cuda")
    fn = L.lapy_tria_divergence if npe == 3 else L.lapy_tet_divergence
    _lib.check(fn(dptr(md.v), md.coords_f32, dptr(md.t), md.m, md.n, dptr(pat.diag_pos), dptr(pat.seg_ptr),
                  dptr(pat.seg_src), dptr(g), nf, dptr(out), dptr(work), stream()), "divergence")
    return out


def _normalize_dev(g: torch.Tensor) -> None:
    L = _lib.lib()
    _lib.check(L.lapy_normalize_rows3(g.numel() // 3, 0, dptr(g), stream()), "normalize_rows3")


def compute_gradient(geom, vfunc):
    """Per-element gradient: (m, 3) for 1-D ``vfunc``, (m, F, 3) for 2-D."""
    require_cuda()
    vfunc = np.asarray(vfunc)
    scalar = vfunc.ndim == 1
    f = torch.from_numpy(np.ascontiguousarray(vfunc.reshape(vfunc.shape[0], -1), dtype=np.float64)).to("cuda")
    g = _gradient_dev(geom, f).cpu().numpy()
    return g[:, 0, :] if scalar else g


def compute_divergence(geom, tfunc):
    """Integrated divergence at vertices: (n,) for (m, 3) input, (n, F) for (m, F, 3)."""
    require_cuda()
    tfunc = np.asarray(tfunc)
    scalar = tfunc.ndim == 2
    g = torch.from_numpy(np.ascontiguousarray(tfunc.reshape(tfunc.shape[0], -1, 3), dtype=np.float64)).to("cuda")
    d = _divergence_dev(geom, g).cpu().numpy()
    return d[:, 0] if scalar else d


def compute_geodesic_f(geom, vfunc, use_cholmod: bool = False):
    """Function with unit gradient (geodesic distance) from a heat solution.

    gradient -> normalise -> integrated divergence stay on the device; then
    ``Solver(lump=True)`` with ``mass = I`` solves the Poisson problem and the
    minimum is subtracted (diffgeo.py:147-165)."""
    from .solver import Solver

    require_cuda()
    vfunc = np.asarray(vfunc)
    scalar = vfunc.ndim == 1
    f = torch.from_numpy(np.ascontiguousarray(vfunc.reshape(vfunc.shape[0], -1), dtype=np.float64)).to("cuda")
    g = _gradient_dev(geom, f)
    _normalize_dev(g)
    divf = _divergence_dev(geom, g)
    fem = Solver(geom, lump=True, use_cholmod=use_cholmod)
    fem.mass = sparse.eye(fem._A.n, dtype=np.float64)
    vf = fem.poisson(divf.cpu().numpy())
    if scalar:
        vf = vf.reshape(-1)
        return vf - vf.min()
    return vf - vf.min(axis=0)
