"""Anisotropic Laplace-Beltrami (lapy/solver.py:196-308 with the curvature
frame of lapy/tria_mesh.py:1078-1279) against the reference's own outputs
(tests/golden/ref_aniso.npz, made by make_golden_aniso.py): the oracle's
curvature frame and anisotropic assembly (CPU), the GPU curvature frame, and
the GPU assembly through ``Solver(mesh, aniso=...)``, whose frame is computed
on the device."""

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


def _check_frame(ref, name, tri, vtx=None, exact_sign=False):
    u1, u2, c1, c2 = tri
    for val, key in ((c1, "cmin"), (c2, "cmax")):
        r = ref[f"{name}_tri_{key}"]
        np.testing.assert_allclose(val, r, rtol=0, atol=1e-10 * np.abs(r).max())
    if exact_sign:  # the triangle frame itself, sign included
        np.testing.assert_allclose(u1, ref[f"{name}_tri_umin"], rtol=0, atol=1e-10)
        np.testing.assert_allclose(u2, ref[f"{name}_tri_umax"], rtol=0, atol=1e-10)
    assert _same_direction(u1, ref[f"{name}_tri_umin"]) and _same_direction(u2, ref[f"{name}_tri_umax"])
    if vtx is not None:
        for val, key in zip(vtx, ("umin", "umax", "cmin", "cmax", "cmean", "cgauss", "normals")):
            r = ref[f"{name}_vtx_{key}"]
            if val.ndim == 2:
                assert _same_direction(val, r), key
            else:
                np.testing.assert_allclose(val, r, rtol=0, atol=1e-10 * np.abs(r).max())


@pytest.mark.parametrize("name", ["d3", "d4"])
def test_oracle_curvature_frame_matches_reference(ref, name):
    from oracle import curvature as C

    v, t = ref[f"{name}_v"], ref[f"{name}_t"]
    _check_frame(ref, name, C.curvature_tria(v, t, 3), C.curvature(v, t, 3) if name == "d3" else None,
                 exact_sign=True)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["d3", "d4"])
def test_gpu_curvature_frame_matches_reference(cuda_ok, ref, name):
    """The device frame, sign included: the per-vertex 3 x 3 eigenvectors
    come out with LAPACK's signs, which the triangle pooling depends on."""
    from lapy_gb300 import TriaMesh

    mesh = TriaMesh(ref[f"{name}_v"], ref[f"{name}_t"])
    _check_frame(ref, name, mesh.curvature_tria(3), mesh.curvature(3) if name == "d3" else None, exact_sign=True)


@pytest.mark.gpu
def test_gpu_curvature_matches_oracle_on_larger_meshes(cuda_ok):
    from lapy_gb300 import meshes
    from oracle import curvature as C

    for level, seed, smooth in ((5, 11, 10), (4, 3, 0)):
        m = meshes.sh_deform(meshes.icosphere(level), seed=seed)
        got = m.curvature_tria(smooth)
        want = C.curvature_tria(np.asarray(m.v), np.asarray(m.t), smooth)
        for g, w in zip(got, want):
            np.testing.assert_allclose(g, w, rtol=0, atol=1e-9 * max(1.0, np.abs(w).max()))


def test_oracle_curvature_needs_an_oriented_mesh(ref):
    from oracle import curvature as C

    t = ref["d3_t"].copy()
    t[0] = t[0, [0, 2, 1]]
    with pytest.raises(ValueError, match="oriented"):
        C.curvature_tria(ref["d3_v"], t)


@pytest.mark.gpu
def test_gpu_curvature_needs_an_oriented_mesh(cuda_ok, ref):
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
    """Solver(mesh, aniso=...) with this package's own TriaMesh: the device
    curvature frame feeds the GPU anisotropic assembly kernel."""
    from lapy_gb300 import Solver, TriaMesh

    mesh = TriaMesh(ref[f"{name}_v"], ref[f"{name}_t"])
    fem = Solver(mesh, lump=lump, aniso=aniso, aniso_smooth=3)
    for mat, key in ((fem.stiffness, "A"), (fem.mass, "M")):
        r = _csr(ref, f"{name}_{tag}_lump{int(lump)}_{key}")
        assert mat.shape == r.shape
        assert abs(sparse.csc_matrix(mat) - r).max() <= 1e-12 * abs(r).max(), key
