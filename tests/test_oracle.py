"""The oracle against the reference's own outputs (CPU only).

The fixtures under tests/golden were produced by running the reference
(tests/golden/make_golden.py); these tests pin the oracle to them, and the
fixtures to the golden values of the reference's own test suite
(lapy/utils/tests/expected_outcomes.json)."""

from __future__ import annotations

import numpy as np
import pytest
from scipy import sparse

import oracle
from conftest import CASES, csr_from, load_case


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("lump", [False, True])
def test_assembly_matches_reference_bitwise(name, lump):
    d = load_case(name)
    A, M = oracle.assemble_scipy(d["v"], d["t"].astype(np.int64), lump=lump)
    RA, RM = csr_from(d, f"A_lump{int(lump)}"), csr_from(d, f"M_lump{int(lump)}")
    for X, R in ((A, RA), (M, RM)):
        X = X.tocsc()
        X.sort_indices()
        assert np.array_equal(X.indptr, R.indptr) and np.array_equal(X.indices, R.indices)
        assert np.array_equal(X.data, R.data)


@pytest.mark.parametrize("name", CASES)
def test_sorted_sum_order_matches_reference(name):
    """The GPU's (row, col, element) summation order: same pattern, values rel <= 1e-12."""
    d = load_case(name)
    A, M = oracle.assemble_sorted(d["v"], d["t"].astype(np.int64), lump=False)
    RA, RM = csr_from(d, "A_lump0"), csr_from(d, "M_lump0")
    for X, R in ((A, RA), (M, RM)):
        assert np.array_equal(X.indptr, R.indptr) and np.array_equal(X.indices, R.indices)
        floor = 1e-12 * np.abs(R.data).max()
        np.testing.assert_allclose(X.data, R.data, rtol=1e-12, atol=floor)
    _, Ml = oracle.assemble_sorted(d["v"], d["t"].astype(np.int64), lump=True)
    np.testing.assert_allclose(Ml, csr_from(d, "M_lump1").diagonal(), rtol=1e-14)


@pytest.mark.parametrize("name", CASES)
def test_symmetry_and_row_sums(name):
    d = load_case(name)
    A = csr_from(d, "A_lump0")
    if d["t"].shape[1] == 3:
        assert (A != A.T).nnz == 0  # test_TriaMesh_Geodesics.py:62-66 asserts exact symmetry
    else:
        # SciPy sums the duplicates of (i, j) and (j, i) in different orders, so
        # the reference's tetrahedral A is symmetric only to rounding
        assert abs(A - A.T).max() <= 1e-15 * np.abs(A.data).max()
    Xs, _ = oracle.assemble_sorted(d["v"], d["t"].astype(np.int64))
    assert (Xs != Xs.T).nnz == 0  # the (row, col, element) order is exactly symmetric
    rs = np.abs(A.sum(axis=1)).max()
    tol = 1e-5 if d["v"].dtype == np.float32 else 1e-12
    assert rs <= tol * np.abs(A.data).max()


@pytest.mark.parametrize("name", CASES)
def test_eigs_match_reference(name):
    d = load_case(name)
    t = d["t"].astype(np.int64)
    k = int(d["eigs_k"])
    for lump, key in ((False, "evals"), (True, "evals_lump")):
        A, M = oracle.assemble_scipy(d["v"], t, lump=lump)
        ref = d[key]
        scale = np.abs(ref[1])
        if name in ("deformed3", "kuhn5"):
            # no exact degeneracy: the reference's single-vector eigsh is reliable here
            ev, _ = oracle.eigs(A, M, k=k, v0=np.random.default_rng(7).standard_normal(A.shape[0]))
            np.testing.assert_allclose(ev, ref, rtol=1e-9, atol=1e-9 * scale)
        # Symmetric meshes (icosphere, cube, square) have exactly degenerate
        # groups that a single-vector Krylov space can miss (even with a seeded
        # start vector), so the dense solve is the comparison there.
        evd, _ = oracle.eigs_dense(A, M, k=k)
        np.testing.assert_allclose(evd, ref, rtol=1e-9, atol=1e-9 * scale)


@pytest.mark.parametrize("name", CASES)
def test_heat_poisson_geodesic_match_reference(name):
    d = load_case(name)
    v, t = d["v"], d["t"].astype(np.int64)
    np.testing.assert_allclose(oracle.avg_edge_length(v, t), d["avg_edge"], rtol=1e-12)
    u = oracle.diffusion(v, t, 0, m=1.0)
    np.testing.assert_allclose(u, d["heat0"], rtol=1e-10, atol=1e-14 * np.abs(u).max())
    um = oracle.diffusion(v, t, [np.array([0]), np.array([1, 2])], m=1.0)
    np.testing.assert_allclose(um, d["heat_multi"], rtol=1e-10, atol=1e-14 * np.abs(um).max())
    A, M = oracle.assemble_scipy(v, t, lump=True)
    dtup = (np.array([0, 1]), np.array([0.0, 0.5]))
    x = oracle.poisson(A, M, d["evecs_lump"][:, 1], dtup=dtup)
    np.testing.assert_allclose(x, d["poisson_dir"], rtol=1e-8, atol=1e-10 * np.abs(x).max())
    g = (oracle.tria_gradient if t.shape[1] == 3 else oracle.tet_gradient)(v, t, d["heat0"])
    np.testing.assert_allclose(g, d["grad_heat0"], rtol=1e-12, atol=1e-14 * np.abs(g).max())
    dv = (oracle.tria_divergence if t.shape[1] == 3 else oracle.tet_divergence)(v, t, g)
    np.testing.assert_allclose(dv, d["div_grad_heat0"], rtol=1e-10, atol=1e-12 * np.abs(dv).max())
    for scaled in (False, True):
        gf = oracle.geodesic_f(v, t, d["heat0"], scaled=scaled)
        np.testing.assert_allclose(gf, d["geodesic0"], rtol=1e-7, atol=1e-8 * np.abs(gf).max())
    # the consistent Neumann solve agrees with the reference's singular LU to the
    # accuracy that LU reaches (2e-5 on the float32 cube surface)
    gc = oracle.geodesic_f(v, t, d["heat0"], consistent=True)
    np.testing.assert_allclose(gc, d["geodesic0"], rtol=0, atol=1e-4 * np.abs(gc).max())


def test_fixture_pins_reference_golden_values():
    """expected_outcomes.json of the reference's test suite (test_visualization_meshes.py:38-120)."""
    cube = load_case("cubetria")
    assert cube["v"].shape == (2402, 3) and cube["t"].shape == (4800, 3)
    np.testing.assert_allclose(cube["evals"][:3], [-4.17232603e-06, 4.16968140e00, 4.17050233e00],
                               rtol=1e-5, atol=1e-5)
    tet = load_case("cubetetra")
    assert tet["v"].shape == (9261, 3) and tet["t"].shape == (48000, 4)
    np.testing.assert_allclose(tet["evals"], [8.4652565e-05, 9.889787, 9.889887], rtol=1e-4, atol=1e-4)
    # compute_shapedna on cubeTria (test_shape_DNA.py:24-42) agrees at atol 1e-4
    np.testing.assert_allclose(cube["evals"][:3], [-4.0165149e-05, 4.169641, 4.1704664], atol=1e-4)


def test_oracle_cubetetra_eigs():
    tet = load_case("cubetetra")
    A, M = oracle.assemble_scipy(tet["v"], tet["t"].astype(np.int64), lump=False)
    ev, _ = oracle.eigs(A, M, k=3)
    np.testing.assert_allclose(ev, [8.4652565e-05, 9.889787, 9.889887], atol=1e-4)


def test_normalize_scaled_equals_plain_in_range():
    rng = np.random.default_rng(0)
    g = rng.standard_normal((100, 3))
    g[3] = 0.0
    np.testing.assert_allclose(oracle.normalize_rows(g, True), oracle.normalize_rows(g, False), rtol=1e-15, atol=1e-16)
    tiny = g * 1e-200
    plain = oracle.normalize_rows(tiny, False)
    # the reference's form: the squares underflow, x/0 = inf, nan_to_num -> +-1.8e308
    assert np.all(np.abs(plain[~np.all(g == 0, axis=1)]) == np.finfo(np.float64).max)
    np.testing.assert_allclose(oracle.normalize_rows(tiny, True), oracle.normalize_rows(g, True), rtol=1e-14)


def test_csr_sorted_sum_edge_cases():
    # duplicate (i, j) pairs summed in order; an unreferenced middle vertex leaves an empty row
    i = np.array([0, 0, 2, 2, 0])
    j = np.array([0, 2, 2, 0, 0])
    vals = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    X = oracle.csr_sorted_sum(i, j, vals, 3)
    ref = sparse.csr_matrix((vals, (i, j)), shape=(3, 3))
    assert np.array_equal(X.toarray(), ref.toarray())
    assert X.indptr.tolist() == [0, 2, 2, 4]
