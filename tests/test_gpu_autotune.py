"""Autotuned eigensolver settings on the GPU: every knob changes only the
time, so a batch solved with non-default knobs (larger aggregates, looser
refinement rounds, fewer CTAs per SM, reduction folding forced on) has the
same eigenvalues as with the defaults, to the eigenvalue tolerance (rel
1e-8); and a calibration stores a choice that later batches of the same shape
class receive."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch():
    from lapy_gb300 import meshes

    return meshes.deformed_icospheres([3, 4, 3, 5, 4, 3], [901 + i for i in range(6)])


def test_tuned_and_default_settings_agree(cuda_ok):
    from lapy_gb300 import shapedna

    ms = _batch()
    fem = shapedna.BatchedFEM(ms)
    ev0, _, info0 = fem.eigs(k=30, block=4)
    tuned = {"agg_target": 96, "round_rtol": 3e-3, "ctas_per_sm": 4, "fold_pieces": 1, "fold_aggs": 1}
    for block in (2, 8):
        ev1, _, info1 = fem.eigs(k=30, block=block, tuning=tuned)
        assert all(int(s) == 0 for s in info0["status"]) and all(int(s) == 0 for s in info1["status"])
        a, b = ev0.cpu().numpy(), ev1.cpu().numpy()
        np.testing.assert_allclose(b[:, 1:], a[:, 1:], rtol=1e-8)
        assert np.all(np.abs(b[:, 0] - a[:, 0]) <= 1e-8 * a[:, 1])


def test_calibration_is_cached_and_reused(cuda_ok, tmp_path, monkeypatch):
    from lapy_gb300 import autotune, shapedna

    monkeypatch.setenv("LAPY_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    ms = _batch()
    cands = {"block": [4, 2], "round_rtol": [1e-3, 3e-3]}
    choice, report = autotune.calibrate(ms, k=12, sample=4, candidates=cands)
    assert len(report) == 3 and all(np.isfinite(t) for _, t in report)
    got = autotune.choice_for(ms, 12)
    assert got == dict(autotune.DEFAULT, **choice)
    out = shapedna.compute_shapedna_batch(ms, k=12, tuning="auto", return_vectors=False)
    assert len(out) == len(ms) and all(len(o["Eigenvalues"]) == 12 for o in out)
