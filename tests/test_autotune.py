"""Host logic of the eigensolver autotuner (CPU): coordinate descent, the
shape classes, the stratified calibration sample and the persistent cache."""

from __future__ import annotations

import numpy as np

from lapy_gb300 import autotune


def test_descend_keeps_the_fastest_by_a_margin():
    cost = {"block": {4: 1.0, 2: 1.4, 8: 0.8}, "agg_target": {64: 0.0, 96: -0.1},
            "round_rtol": {1e-3: 0.0, 3e-3: -0.01}, "ctas_per_sm": {5: 0.0, 4: 0.2}}

    def measure(c):
        return sum(cost[k][c[k]] for k in cost)

    choice, report = autotune.descend(measure)
    assert choice["block"] == 8 and choice["agg_target"] == 96
    assert choice["round_rtol"] == 1e-3  # 0.01 s of 0.7 s is below the 3 % margin
    assert choice["ctas_per_sm"] == 5
    assert report[0][0] == autotune.DEFAULT and len(report) == 1 + 2 + 1 + 1 + 1


def test_failed_trials_are_never_chosen():
    def measure(c):
        return float("inf") if c["block"] == 2 else 1.0 / c["block"]

    choice, _ = autotune.descend(measure)
    assert choice["block"] == 8


def test_shape_class_and_sample():
    seg = np.cumsum([0, 642, 2562, 40962, 10242, 642, 40962])
    assert autotune.shape_class(seg, 50) == "k50-meshes8-med8192-max65536"
    idx = autotune.stratified_sample(seg, 3)
    sizes = np.diff(seg)
    assert len(idx) == 3 and sizes[idx].max() == sizes.max() and sizes[idx].min() == sizes.min()
    assert autotune.stratified_sample(seg, 32) == list(range(6))


def test_cache_round_trip(tmp_path):
    path = tmp_path / "tune.json"
    c = autotune.TuneCache(path)
    assert c.get("dev", "shape") is None
    c.put("dev", "shape", {"block": 8, "agg_target": 96}, [{"choice": {"block": 8}, "seconds": 1.0}])
    again = autotune.TuneCache(path)
    assert again.get("dev", "shape") == {"block": 8, "agg_target": 96}
    assert again.get("other", "shape") is None
    assert autotune.solver_tuning({"block": 8, "agg_target": 96, "round_rtol": 3e-3}) == \
        {"agg_target": 96, "round_rtol": 3e-3}


class _FakeFem:
    """Stands for a BatchedFEM: rejects an aggregate size, fails a block width."""

    def __init__(self):
        self.calls = []

    def eigs(self, k, block, tuning):
        self.calls.append((block, dict(tuning)))
        if tuning.get("agg_target") == 48:
            raise ValueError("eigs_shift_invert: invalid argument (agg_target)")
        return None, None, {"status": [0, -3] if block == 2 else [0, 0]}


def test_timed_trial_rejected_and_failed_choices_are_infinite():
    fem = _FakeFem()
    assert autotune.timed_trial(fem, 50, dict(autotune.DEFAULT, agg_target=48)) == float("inf")
    assert autotune.timed_trial(fem, 50, dict(autotune.DEFAULT, block=2)) == float("inf")
    t = autotune.timed_trial(fem, 50, dict(autotune.DEFAULT), repeats=3)
    assert 0.0 <= t < 1.0
    # the solver sees only its own knobs (block goes by argument)
    assert all("block" not in tn for _, tn in fem.calls)
