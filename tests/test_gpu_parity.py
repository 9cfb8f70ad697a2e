"""CUDA path against the oracle and the reference's own outputs (GPU).

Tolerances are those the path promises: assembled matrices entrywise rel
<= 1e-12 (indices bit-exact), eigenvalues rel <= 1e-8 (the zero eigenvalue
absolute, relative to lambda_1), eigenvector subspace angles <= 1e-6 over
complete degenerate groups, heat / Poisson / geodesic M-norm rel <= 1e-8."""

from __future__ import annotations

import numpy as np
import pytest
from scipy import sparse

import oracle
from conftest import CASES, csr_from, load_case

pytestmark = pytest.mark.gpu


def _mesh(d):
    from lapy_gb300 import TetMesh, TriaMesh

    t = d["t"]
    return TriaMesh(d["v"], t) if t.shape[1] == 3 else TetMesh(d["v"], t)


def _mnorm_rel(x, ref, mdiag):
    x = x.reshape(len(mdiag), -1)
    ref = ref.reshape(len(mdiag), -1)
    num = np.sqrt(np.sum(mdiag[:, None] * (x - ref) ** 2, axis=0))
    den = np.sqrt(np.sum(mdiag[:, None] * ref ** 2, axis=0))
    return np.max(num / den)


def _groups(ev, rel=1e-6):
    """Index ranges of (near-)degenerate eigenvalue groups."""
    out, start = [], 0
    for i in range(1, len(ev) + 1):
        if i == len(ev) or abs(ev[i] - ev[i - 1]) > rel * max(abs(ev[i - 1]), 1.0):
            out.append((start, i))
            start = i
    return out


def _subspace_angle(X, Y, M):
    """Largest principal angle between span(X) and span(Y) in the M inner product."""
    def mqr(Z):
        G = Z.T @ (M @ Z)
        L = np.linalg.cholesky(0.5 * (G + G.T))
        return np.linalg.solve(L, Z.T).T
    Qx, Qy = mqr(X), mqr(Y)
    s = np.linalg.svd(Qx.T @ (M @ Qy), compute_uv=False)
    return float(np.sqrt(max(0.0, 1.0 - s.min() ** 2)))


def _check_eigs(ev, V, ref_ev, ref_V, M, complete_upto=None):
    lam1 = abs(ref_ev[1])
    assert abs(ev[0] - ref_ev[0]) <= 1e-8 * lam1
    np.testing.assert_allclose(ev[1:], ref_ev[1:], rtol=1e-8)
    # compare complete groups only
    groups = _groups(ref_ev)
    if complete_upto is not None:
        groups = [g for g in groups if g[1] <= complete_upto]
    else:
        groups = groups[:-1]  # the last group may be cut by k
    for a, b in groups:
        assert _subspace_angle(V[:, a:b], ref_V[:, a:b], M) <= 1e-6, (a, b)
    G = V.T @ (M @ V)
    np.testing.assert_allclose(G, np.eye(G.shape[0]), atol=1e-9)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("lump", [False, True])
def test_assembly_parity(cuda_ok, name, lump):
    from lapy_gb300 import Solver

    d = load_case(name)
    fem = Solver(_mesh(d), lump=lump)
    A, M = fem.stiffness, fem.mass
    RA, RM = csr_from(d, f"A_lump{int(lump)}"), csr_from(d, f"M_lump{int(lump)}")
    assert np.array_equal(A.indptr, RA.indptr) and np.array_equal(A.indices, RA.indices)
    np.testing.assert_allclose(A.data, RA.data, rtol=1e-12, atol=1e-12 * np.abs(RA.data).max())
    np.testing.assert_allclose(M.toarray(), RM.toarray(), rtol=1e-12, atol=1e-14 * np.abs(RM.data).max())
    # the GPU sums in the oracle's deterministic order: bit-identical values
    SA, SM = oracle.assemble_sorted(d["v"], d["t"].astype(np.int64), lump=lump)
    assert np.array_equal(A.data, SA.data)
    if lump:
        assert np.array_equal(M.diagonal(), SM)
    else:
        assert np.array_equal(M.data, SM.data)
    assert A.getformat() == "csc"
    assert (A != A.T).nnz == 0


@pytest.mark.parametrize("name", ["square", "kuhn5"])
def test_assembly_float32_output(cuda_ok, name):
    from lapy_gb300 import Solver

    d = load_case(name)
    fem = Solver(_mesh(d), lump=False, dtype=np.float32)
    A32, _ = oracle.assemble_scipy(d["v"], d["t"].astype(np.int64), dtype=np.float32)
    assert fem.stiffness.dtype == np.float32
    np.testing.assert_allclose(fem.stiffness.toarray(), A32.toarray(), rtol=1e-6, atol=1e-6 * abs(A32).max())


@pytest.mark.parametrize("name", CASES)
def test_avg_edge_length(cuda_ok, name):
    d = load_case(name)
    rtol = 1e-6 if d["v"].dtype == np.float32 else 1e-13
    np.testing.assert_allclose(_mesh(d).avg_edge_length(), d["avg_edge"], rtol=rtol)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("lump", [False, True])
def test_eigs_parity(cuda_ok, name, lump):
    from lapy_gb300 import Solver

    d = load_case(name)
    fem = Solver(_mesh(d), lump=lump)
    k = int(d["eigs_k"])
    ev, V = fem.eigs(k=k)
    A, M = oracle.assemble_scipy(d["v"], d["t"].astype(np.int64), lump=lump)
    ref_ev, ref_V = oracle.eigs_dense(A, M, k=k + 6)
    _check_eigs(ev, V, ref_ev[:k], ref_V[:, :k], sparse.csr_matrix(M))
    np.testing.assert_allclose(ev[1:], d["evals_lump" if lump else "evals"][1:], rtol=1e-8)


def test_eigs_k50_cuts_degenerate_groups(cuda_ok):
    """ico L3, k=50: groups of the icosahedral spectrum straddle k."""
    from lapy_gb300 import Solver, meshes

    mesh = meshes.icosphere(3)
    fem = Solver(mesh, lump=False)
    ev, V = fem.eigs(k=50)
    A, M = oracle.assemble_scipy(mesh.v, mesh.t)
    ref_ev, ref_V = oracle.eigs_dense(A, M, k=60)
    groups = _groups(ref_ev)
    complete = max(b for a, b in groups if b <= 50)
    _check_eigs(ev, V, ref_ev[:50], ref_V[:, :50], sparse.csr_matrix(M), complete_upto=complete)


def test_eigs_tet_kuhn(cuda_ok):
    from lapy_gb300 import Solver, meshes

    mesh = meshes.kuhn_cube(10, jitter=0.2, seed=4)
    fem = Solver(mesh, lump=False)
    ev, V = fem.eigs(k=20)
    A, M = oracle.assemble_scipy(mesh.v, mesh.t)
    ref_ev, ref_V = oracle.eigs_dense(A, M, k=24)
    _check_eigs(ev, V, ref_ev[:20], ref_V[:, :20], sparse.csr_matrix(M))


def test_eigs_deformed_l5_k50_against_eigsh(cuda_ok):
    """Icosphere-L5-sized (10,242 vertices) deformed sphere, k=50 vs the reference method (eigsh + splu)."""
    from lapy_gb300 import Solver, meshes

    mesh = meshes.sh_deform(meshes.icosphere(5), seed=21)
    fem = Solver(mesh, lump=False)
    ev, V = fem.eigs(k=50)
    A, M = oracle.assemble_scipy(mesh.v, mesh.t)
    ref_ev, ref_V = oracle.eigs(A, M, k=50, v0=np.random.default_rng(3).standard_normal(A.shape[0]))
    _check_eigs(ev, V, ref_ev, ref_V, sparse.csr_matrix(M))


def test_batched_eigs_matches_single(cuda_ok):
    from lapy_gb300 import meshes, shapedna

    ms = [meshes.sh_deform(meshes.icosphere(lv), seed=s) for lv, s in ((2, 1), (3, 2), (2, 3), (3, 4))]
    out = shapedna.compute_shapedna_batch(ms, k=12, block=2)
    for mesh, res in zip(ms, out):
        A, M = oracle.assemble_scipy(mesh.v, mesh.t)
        ref_ev, ref_V = oracle.eigs_dense(A, M, k=12)
        _check_eigs(res["Eigenvalues"], res["Eigenvectors"], ref_ev, ref_V, sparse.csr_matrix(M),
                    complete_upto=12)
        assert res["DoF"] == len(mesh.v) and res["NumEW"] == 12


@pytest.mark.parametrize("name", CASES)
def test_heat_parity(cuda_ok, name):
    from lapy_gb300 import heat

    d = load_case(name)
    mesh = _mesh(d)
    mdiag = csr_from(d, "M_lump1").diagonal()
    u = heat.diffusion(mesh, 0, m=1.0)
    assert u.shape == (len(d["v"]),)
    # float32 coordinates: t = m * h^2 is summed in a different order than NumPy
    tol = 1e-6 if d["v"].dtype == np.float32 else 1e-8
    assert _mnorm_rel(u, d["heat0"], mdiag) <= tol
    um = heat.diffusion(mesh, [np.array([0]), np.array([1, 2])], m=1.0)
    assert um.shape == (len(d["v"]), 2)
    assert _mnorm_rel(um, d["heat_multi"], mdiag) <= tol
    # one- and multi-column solves stop at different iterates of the same tolerance
    np.testing.assert_allclose(um[:, 0], u, rtol=1e-7, atol=1e-10 * np.abs(u).max())


def test_heat_batch_matches_oracle(cuda_ok):
    """Batched heat: every mesh its own t = avg_edge_length**2 and seed vertex."""
    from lapy_gb300 import heat, meshes

    ms = [meshes.sh_deform(meshes.icosphere(lv), seed=s) for lv, s in ((2, 5), (3, 6), (1, 7), (3, 8), (2, 9))]
    vids = [0, 11, 3, 40, 7]
    out = heat.diffusion_batch(ms, vids, m=2.0)
    for mesh, v, u in zip(ms, vids, out):
        ref = oracle.diffusion(mesh.v, mesh.t, v, m=2.0)
        _, M = oracle.assemble_scipy(mesh.v, mesh.t, lump=True)
        assert u.shape == (len(mesh.v),)
        assert _mnorm_rel(u, ref, M.diagonal()) <= 1e-8
    with pytest.raises(ValueError, match="out-of-range"):
        heat.diffusion_batch(ms, [0, 0, 0, 0, len(ms[4].v)])
    with pytest.raises(ValueError, match="one vertex per mesh"):
        heat.diffusion_batch(ms, [0, 1])


def test_heat_out_of_range_raises(cuda_ok):
    from lapy_gb300 import heat

    d = load_case("square")
    mesh = _mesh(d)
    with pytest.raises(ValueError, match="out-of-range"):
        heat.diffusion(mesh, np.array([len(mesh.v)]), m=1)
    with pytest.raises(ValueError, match="out-of-range"):
        heat.diffusion(mesh, [np.array([0]), np.array([len(mesh.v)])], m=1)


@pytest.mark.parametrize("name", CASES)
def test_poisson_parity(cuda_ok, name):
    from lapy_gb300 import Solver

    d = load_case(name)
    fem = Solver(_mesh(d), lump=True)
    mdiag = csr_from(d, "M_lump1").diagonal()
    dtup = (np.array([0, 1]), np.array([0.0, 0.5]))
    x = fem.poisson(d["evecs_lump"][:, 1], dtup=dtup)
    assert x.shape == (len(d["v"]),)
    assert _mnorm_rel(x, d["poisson_dir"], mdiag) <= 1e-8
    x2 = fem.poisson(d["evecs_lump"][:, 1:4], dtup=dtup)
    assert x2.shape == (len(d["v"]), 3)
    assert _mnorm_rel(x2, d["poisson_dir_2d"], mdiag) <= 1e-8
    # 2-D rhs equals column-wise 1-D solves (test_solver.py:25-58)
    for c in range(3):
        np.testing.assert_allclose(x2[:, c], fem.poisson(d["evecs_lump"][:, 1 + c], dtup=dtup), rtol=1e-6, atol=1e-9)
    assert fem.poisson(0.0).ndim == 1


def test_poisson_validation(cuda_ok):
    from lapy_gb300 import Solver

    fem = Solver(_mesh(load_case("square")), lump=True)
    with pytest.raises(ValueError, match="dtup indices need to be unique"):
        fem.poisson(0.0, dtup=(np.array([0, 0]), np.array([0.0, 1.0])))
    with pytest.raises(ValueError, match="h should be either scalar"):
        fem.poisson(np.zeros(3))
    with pytest.raises(ValueError, match="ntup should contain"):
        fem.poisson(0.0, ntup=(np.array([0]), np.array([1.0, 2.0])))


@pytest.mark.parametrize("name", CASES)
def test_gradient_divergence_geodesic(cuda_ok, name):
    from lapy_gb300 import diffgeo

    d = load_case(name)
    mesh = _mesh(d)
    g = diffgeo.compute_gradient(mesh, d["heat0"])
    np.testing.assert_allclose(g, d["grad_heat0"], rtol=1e-12, atol=1e-14 * np.abs(g).max())
    dv = diffgeo.compute_divergence(mesh, d["grad_heat0"])
    np.testing.assert_allclose(dv, d["div_grad_heat0"], rtol=1e-10, atol=1e-12 * np.abs(dv).max())
    gf = diffgeo.compute_geodesic_f(mesh, d["heat0"])
    mdiag = csr_from(d, "M_lump1").diagonal()
    # the oracle's consistent Neumann solve is the comparison at 1e-8; the
    # reference's singular LU differs from it by up to 2e-5 on the float32
    # fixture meshes (an inconsistent right-hand side amplified by a near-zero
    # pivot), so the reference's output is met at that level
    ref = oracle.geodesic_f(d["v"], d["t"].astype(np.int64), d["heat0"], consistent=True)
    assert _mnorm_rel(gf, ref, mdiag) <= 1e-8
    assert _mnorm_rel(gf, d["geodesic0"], mdiag) <= 1e-4
    # 2-D input equals column-wise 1-D (test_diffgeo.py:53-227)
    f2 = np.column_stack((d["heat0"], d["heat_multi"][:, 1]))
    g2 = diffgeo.compute_gradient(mesh, f2)
    np.testing.assert_allclose(g2[:, 0, :], g, rtol=1e-12, atol=0)
    gf2 = diffgeo.compute_geodesic_f(mesh, f2)
    np.testing.assert_allclose(gf2[:, 0], gf, rtol=1e-7, atol=1e-9 * np.abs(gf).max())


def test_solver_api_surface(cuda_ok):
    from lapy_gb300 import Solver, meshes

    mesh = meshes.icosphere(2)
    fem = Solver(mesh, lump=True)
    B = fem.mass
    assert B.sum() == pytest.approx(4 * np.pi, rel=2e-2)
    Bi = B.copy()
    Bi.data **= -1
    assert Bi is not B
    fem.mass = sparse.eye(fem.stiffness.shape[0])
    x = fem.poisson(np.ones(len(mesh.v)) - 1.0)
    assert np.allclose(x, 0.0)
    with pytest.raises(ValueError, match="unknown"):
        Solver(object())


def test_maxiter_reports_no_convergence(cuda_ok):
    from lapy_gb300 import _device, _lib, meshes, Solver

    fem = Solver(meshes.icosphere(3), lump=True)
    A = fem._A
    b = __import__("torch").ones(A.n, 1, dtype=__import__("torch").float64, device="cuda")
    with pytest.raises(_lib.ConvergenceError):
        _device.pcg_solve(A.indptr, A.indices, A.data, A.n, A.data.numel(), b, rtol=1e-14, maxiter=2, mixed=False)
