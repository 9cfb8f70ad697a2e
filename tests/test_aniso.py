"""Anisotropic Laplace-Beltrami (lapy/solver.py:196-308 with the curvature
frame of lapy/tria_mesh.py:1078-1279) against the reference's own outputs
(tests/golden/ref_aniso.npz, made by make_golden_aniso.py): the host
curvature frame, the oracle's anisotropic assembly, and the GPU assembly
through ``Solver(mesh, aniso=...)``."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
from scipy import sparse

import oracle

GOLD = Path(__file__).resolve().parent / "golden"
CONFIGS = [("d3", "a12", (1.0, 2.0)), ("d3", "a05", 0.5), ("d4", "a12", (1.0, 2.0))]


@pytest.fixture(scope="module")
def ref():
    return np.load(GOLD / "ref_aniso.npz")


def _csr(ref, prefix):
    n = len(ref[f"{prefix}_indptr"]) - 1
    return sparse.csc_matrix((ref[f"{prefix}_data"], ref[f"{prefix}_indices"], ref[f"{prefix}_indptr"]),
                             shape=(n, n))


def _same_direction(u, r, tol=1e-10):
    """Rows agree up to sign (an eigenvector's sign is free)."""
    return np.all(np.abs(np.abs(np.sum(u * r, axis=1)) - 1.0) <= tol)


def _aniso_mat(c1, c2, aniso):
    a0, a1 = aniso if isinstance(aniso, tuple) else (aniso, aniso)
    am = np.empty((len(c1), 2))
    am[:, 1] = np.exp(-a1 * np.abs(c1))
    am[:, 0] = np.exp(-a0 * np.abs(c2))
    return am


@pytest.mark.parametrize("name", ["d3", "d4"])
def test_curvature_frame_matches_reference(ref, name):
    from lapy_gb300 import TriaMesh

    mesh = TriaMesh(ref[f"{name}_v"], ref[f"{name}_t"])
    u1, u2, c1, c2 = mesh.curvature_tria(3)
    for val, key in ((c1, "cmin"), (c2, "cmax")):
        r = ref[f"{name}_tri_{key}"]
        np.testing.assert_allclose(val, r, rtol=0, atol=1e-10 * np.abs(r).max())
    assert _same_direction(u1, ref[f"{name}_tri_umin"]) and _same_direction(u2, ref[f"{name}_tri_umax"])
    if name == "d3":
        vt = mesh.curvature(3)
        for val, key in zip(vt, ("umin", "umax", "cmin", "cmax", "cmean", "cgauss", "normals")):
            r = ref[f"{name}_vtx_{key}"]
            if val.ndim == 2:
                assert _same_direction(val, r), key
            else:
                np.testing.assert_allclose(val, r, rtol=0, atol=1e-10 * np.abs(r).max())


def test_curvature_needs_an_oriented_mesh(ref):
    from lapy_gb300 import TriaMesh

    t = ref["d3_t"].copy()
    t[0] = t[0, [0, 2, 1]]
    with pytest.raises(ValueError, match="oriented"):
        TriaMesh(ref["d3_v"], t).curvature_tria()


@pytest.mark.parametrize("name,tag,aniso", CONFIGS)
@pytest.mark.parametrize("lump", [False, True])
def test_oracle_aniso_assembly_matches_reference(ref, name, tag, aniso, lump):
    v, t = ref[f"{name}_v"], ref[f"{name}_t"]
    u1, u2, c1, c2 = (ref[f"{name}_tri_{k}"] for k in ("umin", "umax", "cmin", "cmax"))
    A, M = oracle.assemble_scipy(v, t, lump=lump, frame=(u1, u2, _aniso_mat(c1, c2, aniso)))
    for mat, key in ((A, "A"), (M, "M")):
        r = _csr(ref, f"{name}_{tag}_lump{int(lump)}_{key}")
        assert abs(mat - r).max() <= 1e-12 * abs(r).max()


@pytest.mark.gpu
@pytest.mark.parametrize("name,tag,aniso", CONFIGS)
@pytest.mark.parametrize("lump", [False, True])
def test_gpu_aniso_solver_matches_reference(cuda_ok, ref, name, tag, aniso, lump):
    """Solver(mesh, aniso=...) with this package's own TriaMesh: the host
    curvature frame feeds the GPU anisotropic assembly kernel."""
    from lapy_gb300 import Solver, TriaMesh

    mesh = TriaMesh(ref[f"{name}_v"], ref[f"{name}_t"])
    fem = Solver(mesh, lump=lump, aniso=aniso, aniso_smooth=3)
    for mat, key in ((fem.stiffness, "A"), (fem.mass, "M")):
        r = _csr(ref, f"{name}_{tag}_lump{int(lump)}_{key}")
        assert mat.shape == r.shape
        assert abs(sparse.csc_matrix(mat) - r).max() <= 1e-12 * abs(r).max(), key
