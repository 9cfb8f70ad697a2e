"""GPU drop-ins for the heat-method geodesic pieces of lapy/diffgeo.py, and
its mean-curvature flow.

``compute_gradient`` (diffgeo.py:26-54), ``compute_divergence`` (:57-85) and
``compute_geodesic_f`` (:116-165) for triangle and tetrahedral meshes, with
1-D or 2-D vertex functions.  The gradient, the normalisation and the
integrated divergence are CUDA kernels; the Poisson step is
``Solver.poisson`` with the identity mass, as in the reference.
``tria_mean_curvature_flow`` (:523-606) repeats the GPU mass assembly and a
three-column PCG solve of (M + step A) per step.
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


def tria_mean_curvature_flow(tria, max_iter: int = 30, stop_eps: float = 1e-13, step: float = 1.0,
                             use_cholmod: bool = False, rtol: float = 1e-12):
    """Non-singular mean-curvature flow (Kazhdan et al. 2012), as
    lapy/diffgeo.py:523-606: the stiffness A of the normalised input mesh is
    kept, and each step assembles the lumped mass M of the current mesh on the
    GPU, solves (M + step A) V = M V for the three coordinate columns with the
    GPU PCG (relative residual ``rtol``; the reference factorises), then
    re-normalises (unit area, centroid at the origin).  Stops after
    ``max_iter`` steps or when sum_k (dv_k' M dv_k)^2 < ``stop_eps``.
    Returns a new TriaMesh."""
    from ._device import DeviceCSR, MeshDevice, assemble, axpby, pcg_solve
    from .solver import Solver, _import_optional
    from .tria_mesh import TriaMesh

    if use_cholmod:
        _import_optional("sksparse")
    require_cuda()
    mesh = TriaMesh(tria.v, tria.t)
    mesh.normalize_()
    fem = Solver(mesh, lump=True)
    A = fem._A.as_f64()
    md, pat = pattern_of(mesh)
    n = A.n
    for _ in range(max_iter):
        v_last = mesh.v
        vd = torch.from_numpy(np.ascontiguousarray(mesh.v, dtype=np.float64)).to("cuda")
        cur = MeshDevice(vd, md.t, md.n, md.nv, md.m, md.npe)
        _, mdiag = assemble(cur, pat, True, torch.float64)
        M = DeviceCSR(n, diag=mdiag)
        mv = M.matmul(vd)
        kv = M.on_pattern(A.indptr, A.indices, A.data.numel())
        axpby(step, A.data.contiguous(), 1.0, kv, out=kv)
        x, _, _ = pcg_solve(A.indptr, A.indices, kv, n, kv.numel(), mv, rtol)
        mesh.v = x.cpu().numpy()
        mesh.normalize_()
        dv = mesh.v - v_last
        mh = mdiag.cpu().numpy()
        diff = np.trace(np.square(dv.T @ (mh[:, np.newaxis] * dv)))
        if diff < stop_eps:
            break
    return mesh
