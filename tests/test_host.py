"""Host-side logic that needs no GPU: meshes, argument checks, dispatch."""

from __future__ import annotations

import numpy as np
import pytest

from lapy_gb300 import TetMesh, TriaMesh, meshes


def test_icosphere_counts():
    for lv in range(4):
        m = meshes.icosphere(lv)
        assert m.v.shape == (10 * 4 ** lv + 2, 3) and m.t.shape == (20 * 4 ** lv, 3)
        np.testing.assert_allclose(np.linalg.norm(m.v, axis=1), 1.0, rtol=1e-15)


def test_icosphere_matches_reference_refinement():
    """refine_ numbering equals the reference's (tria_mesh.py:1452-1487): the
    golden icosphere L3 was produced by the reference's refine_."""
    from conftest import load_case

    d = load_case("ico3")
    m = meshes.icosphere(3)
    assert np.array_equal(m.t, d["t"]) and np.array_equal(m.v, d["v"])


def test_kuhn_cube_counts_and_orientation():
    k = meshes.kuhn_cube(4, jitter=0.2, seed=1)
    assert k.v.shape == (125, 3) and k.t.shape == (384, 4)
    e1, e2, e3 = (k.v[k.t[:, i]] - k.v[k.t[:, 0]] for i in (1, 2, 3))
    vol = np.abs(np.einsum("ij,ij->i", e3, np.cross(e1, e2)))
    assert vol.min() > 0
    assert meshes.kuhn_center_vertex(64) == 32 + 65 * (32 + 65 * 32)


def test_mesh_validation_errors():
    with pytest.raises(ValueError, match="Max index exceeds"):
        TriaMesh(np.zeros((3, 3)), [[0, 1, 3]])
    with pytest.raises(ValueError, match="empty"):
        TriaMesh(np.zeros((3, 3)), np.zeros((0, 3), dtype=int))
    with pytest.raises(ValueError, match="Max index exceeds"):
        TetMesh(np.zeros((4, 3)), [[0, 1, 2, 4]])
    m = TriaMesh(np.array([[0, 0], [1, 0], [0, 1]], dtype=float), [[0, 1, 2]])
    assert m.v.shape == (3, 3) and m.is_2d()


def test_solver_rejects_unknown_geometry_before_gpu():
    from lapy_gb300 import Solver

    class Polygon:  # any other type name
        v = np.zeros((3, 3))
        t = np.zeros((1, 3), dtype=int)

    with pytest.raises(ValueError, match='Geometry type "Polygon" unknown'):
        Solver(Polygon())


def test_solver_aniso_length_check_before_gpu():
    from lapy_gb300 import Solver

    class TriaMesh:  # noqa: D401 - stands in for a mesh with a curvature frame
        t = np.zeros((2, 3), dtype=int)
        v = np.zeros((3, 3))

        def curvature_tria(self, smoothit=3):
            z = np.zeros((2, 3))
            return z, z, np.zeros(2), np.zeros(2)

    with pytest.raises(ValueError, match="length 2"):
        Solver(TriaMesh(), aniso=(1.0, 2.0, 3.0))


def test_heat_seed_range_check_before_gpu():
    from lapy_gb300 import heat

    m = meshes.icosphere(1)
    with pytest.raises(ValueError, match="out-of-range"):
        heat.diffusion(m, [np.array([0]), np.array([10_000])])
    with pytest.raises(ValueError, match="out-of-range"):
        heat.diffusion(m, -1)


def test_sh_deformation_is_deterministic():
    a = meshes.sh_deform(meshes.icosphere(2), seed=3)
    b = meshes.sh_deform(meshes.icosphere(2), seed=3)
    assert np.array_equal(a.v, b.v)
    r = np.linalg.norm(a.v, axis=1)
    assert 0.5 < r.min() < r.max() < 1.5


def test_pcg_warp_plan_is_consistent():
    """The persistent PCG's warp plan (virtual warps and CTAs, per-CTA
    reduction slots, row coverage) on random batches: tiny, empty and large
    segments, and segment lengths that leave short tail units."""
    from lapy_gb300 import _lib

    L = _lib.lib()
    rng = np.random.default_rng(7)
    for trial in range(300):
        nseg = int(rng.integers(1, 40))
        if trial % 4 == 0:
            lens = rng.integers(0, 40, nseg)
        elif trial % 4 == 1:
            lens = rng.integers(0, 3000, nseg)
        else:
            lens = rng.integers(1, 200, nseg) * 32 + rng.integers(0, 2, nseg) * rng.integers(1, 31, nseg)
        if trial % 7 == 0:
            lens[::3] = 0
        seg_row = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
        st = L.lapy_plan_check(seg_row.ctypes.data, nseg)
        assert st == 0, (trial, L.lapy_last_error().decode())
    bad = np.array([0, 10, 5], dtype=np.int32)  # decreasing offsets are rejected
    assert L.lapy_plan_check(bad.ctypes.data, 2) != 0
