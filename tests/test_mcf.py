"""Mean-curvature flow (lapy/diffgeo.py:523-606): the oracle pinned to the
reference's outputs (tests/golden/ref_mcf.npz, made by make_golden_mcf.py),
and the GPU flow (assembly + PCG per step) against the same outputs."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle

GOLD = Path(__file__).resolve().parent / "golden"
CASES = [("mcf5_v", dict(max_iter=5)), ("mcf5_step05_v", dict(max_iter=5, step=0.5)), ("mcf_default_v", {})]


@pytest.fixture(scope="module")
def ref():
    return np.load(GOLD / "ref_mcf.npz")


@pytest.mark.parametrize("key,kw", CASES)
def test_oracle_matches_reference(ref, key, kw):
    v = oracle.mean_curvature_flow(ref["v"], ref["t"], **kw)
    assert np.abs(v - ref[key]).max() <= 1e-12 * np.abs(ref[key]).max()


@pytest.mark.gpu
@pytest.mark.parametrize("key,kw", CASES)
def test_gpu_flow_matches_reference(cuda_ok, ref, key, kw):
    from lapy_gb300 import TriaMesh, diffgeo

    mesh = TriaMesh(ref["v"].copy(), ref["t"].copy())
    out = diffgeo.tria_mean_curvature_flow(mesh, **kw)
    assert type(out).__name__ == "TriaMesh" and out is not mesh
    np.testing.assert_array_equal(mesh.v, ref["v"])  # the input mesh is not modified
    np.testing.assert_array_equal(out.t, ref["t"])
    # PCG to a relative residual of 1e-12 per step instead of the reference's LU
    assert np.abs(out.v - ref[key]).max() <= 1e-8 * np.abs(ref[key]).max()
    # the flow ends on a unit-area surface centred at the origin
    c, area = out.centroid()
    assert abs(area - 1.0) <= 1e-12 and np.abs(c).max() <= 1e-12
