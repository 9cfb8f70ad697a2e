"""The benchmarked configurations against the reference method (GPU).

The batched ShapeDNA workload is measured at block width 4 with the
two-level preconditioner, inner refinement rounds of 1e-3 and a Ritz
tolerance of 1e-8 on meshes up to icosphere level 6.  This file runs that
exact solver configuration on a smaller batch of the same mesh family
(levels 3-6, one level-6 mesh) and holds every mesh to the bars of the
path: eigenvalues rel <= 1e-8 against the reference's own call
(``eigsh`` in shift-invert mode with ``splu(A - sigma M)``,
lapy/solver.py:702-716), lambda_0 absolute <= 1e-8 lambda_1, eigenvector
subspace angles <= 1e-6 over complete groups and M-orthonormality 1e-9.
It also checks the batched assembly's per-mesh element-measure clamp
(lapy/solver.py:158-159) against single-mesh assembly."""

from __future__ import annotations

import numpy as np
import pytest
from scipy import sparse

import oracle
from test_gpu_parity import _check_eigs

pytestmark = pytest.mark.gpu

LEVELS = (3, 4, 5, 6, 3, 4, 5, 4)


def test_batched_headline_configuration(cuda_ok):
    """8 deformed icospheres (levels 3-6), k=50, block 4, two-level, as the benchmark runs it."""
    from lapy_gb300 import meshes, shapedna

    seeds = [2024 * 100003 + i for i in range(len(LEVELS))]
    ms = meshes.deformed_icospheres(list(LEVELS), seeds)
    fem = shapedna.BatchedFEM(ms, lump=False)
    evals, evecs, info = fem.eigs(k=50, block=4, precond="twolevel")
    assert all(int(s) == 0 for s in info["status"])
    ev = evals.cpu().numpy()
    V = evecs.cpu().numpy()
    for i, mesh in enumerate(ms):
        A, M = oracle.assemble_scipy(mesh.v, mesh.t)
        v0 = np.random.default_rng(100 + i).standard_normal(A.shape[0])
        ref_ev, ref_V = oracle.eigs(A, M, k=50, v0=v0)
        r0, r1 = fem.seg_row[i], fem.seg_row[i + 1]
        _check_eigs(ev[i], V[r0:r1], ref_ev, ref_V, sparse.csr_matrix(M))


def _with_degenerate_triangles(mesh, count, scale):
    """The mesh with `count` extra vertices, each a copy of a vertex of an
    existing edge and forming a triangle of exactly zero area on that edge;
    coordinates scaled so that each mesh has its own mean element measure."""
    from lapy_gb300 import TriaMesh

    v = np.asarray(mesh.v, dtype=np.float64) * scale
    t = np.asarray(mesh.t, dtype=np.int64)
    extra_v, extra_t = [], []
    for j in range(count):
        a, b = t[j, 0], t[j, 1]
        extra_v.append(v[a].copy())  # coincides with vertex a: zero area
        extra_t.append([a, b, len(v) + j])
    v2 = np.vstack([v, np.array(extra_v)])
    t2 = np.vstack([t, np.array(extra_t)]).astype(np.int32)
    return TriaMesh(v2, t2)


def test_batched_clamp_is_per_mesh(cuda_ok):
    """Degenerate elements of each mesh get that mesh's own clamp: the batch's
    blocks equal single-mesh assembly to the last bits of the mean measure,
    which the two paths sum in different orders (the clamp enters both the
    mass and the cotangent terms of the degenerate elements)."""
    from lapy_gb300 import Solver, meshes, shapedna

    ms = [_with_degenerate_triangles(meshes.icosphere(2), 3, 1.0),
          _with_degenerate_triangles(meshes.icosphere(3), 2, 40.0),
          meshes.sh_deform(meshes.icosphere(2), seed=9)]
    fem = shapedna.BatchedFEM(ms, lump=False)
    a = fem.a_vals.cpu().numpy()
    m = fem.m_vals.cpu().numpy()
    indptr = fem.indptr.cpu().numpy()
    for i, mesh in enumerate(ms):
        single = Solver(mesh, lump=False)
        A1, M1 = single.stiffness, single.mass
        r0, r1 = fem.seg_row[i], fem.seg_row[i + 1]
        k0, k1 = indptr[r0], indptr[r1]
        np.testing.assert_allclose(a[k0:k1], sparse.csr_matrix(A1).data, rtol=1e-14, atol=0)
        np.testing.assert_allclose(m[k0:k1], sparse.csr_matrix(M1).data, rtol=1e-14, atol=0)
        # the mass carries this mesh's clamp (the oracle's mean is NumPy's)
        Mref = oracle.assemble_sorted(np.asarray(mesh.v), np.asarray(mesh.t))[1]
        np.testing.assert_allclose(m[k0:k1], Mref.data, rtol=1e-14, atol=0)


def test_batch_input_built_on_the_device(cuda_ok):
    """Meshes concatenated into one batch: vertex blocks stacked, element
    indices offset on the device (int64 and int32 inputs), and the reference's
    preconditions checked there (indices inside the mesh, every vertex used)."""
    from lapy_gb300 import TriaMesh, meshes, shapedna

    ms = [meshes.sh_deform(meshes.icosphere(2), seed=1), meshes.icosphere(1), meshes.sh_deform(meshes.icosphere(3), 2)]
    for dt in (np.int64, np.int32):
        batch = [TriaMesh(m.v, np.asarray(m.t, dtype=dt)) for m in ms]
        inp = shapedna.BatchInput(batch)
        off = np.cumsum([0] + [len(m.v) for m in ms])
        want = np.concatenate([np.asarray(m.t) + off[i] for i, m in enumerate(ms)])
        np.testing.assert_array_equal(inp.mesh.t.cpu().numpy(), want)
        np.testing.assert_array_equal(inp.mesh.v.cpu().numpy(), np.concatenate([m.v for m in ms]))
    bad = TriaMesh(ms[1].v, ms[1].t.copy())
    bad.t[0, 0] = len(bad.v)  # outside the mesh
    with pytest.raises(ValueError, match="outside"):
        shapedna.BatchInput([ms[0], bad])
    extra = TriaMesh(np.vstack([ms[1].v, [[0.0, 0.0, 2.0]]]), ms[1].t)  # a vertex no triangle uses
    with pytest.raises(ValueError, match="every vertex"):
        shapedna.BatchInput([ms[0], extra])
