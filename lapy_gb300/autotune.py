"""Autotuner of the batched shift-invert eigensolver.

The reference has nothing to tune (SciPy's ARPACK and SuperLU pick their own
parameters).  The GPU eigensolver has a few knobs whose best values depend on
the device and on the shape of the batch (how many meshes, how large):

* ``block``        Lanczos block width (columns per inner solve): 2, 4 or 8;
* ``agg_target``   rows per aggregate of the two-level coarse space;
* ``round_rtol``   residual reduction of each FP32 refinement round;
* ``ctas_per_sm``  resident CTAs per SM of the persistent PCG.

``calibrate`` times the solver on a stratified sample of the batch (whole
meshes, the largest sizes included) by coordinate descent from the defaults,
one knob at a time in the order above, keeping a candidate only when it is at
least ``margin`` faster.  The choice is stored in a JSON cache keyed by
device (name, SM count, compute capability) and batch shape class (mesh
count, median and largest mesh size, each rounded up to a power of two, and
k), so later batches of the same class reuse it without timing anything:
given a cache, the knobs a batch gets are a pure function of its shape.
Every knob changes only the time to solution; the eigenvalues agree to the
solver's tolerance (``tests/test_gpu_autotune.py``).

The cache lives at ``$LAPY_AUTOTUNE_CACHE`` or
``~/.cache/lapy_gb300/autotune.json``.
"""

from __future__ import annotations

import json
import math
import os
import time
from pathlib import Path

import numpy as np

DEFAULT = {"block": 4, "agg_target": 64, "round_rtol": 1e-3, "ctas_per_sm": 5}
CANDIDATES = {
    "block": [4, 2, 8],
    "agg_target": [64, 96],
    "round_rtol": [1e-3, 3e-3],
    "ctas_per_sm": [5, 4],
}
SOLVER_KEYS = ("agg_target", "round_rtol", "fold_pieces", "fold_aggs", "ctas_per_sm")


def _pow2(x: float) -> int:
    return 1 << max(0, int(math.ceil(math.log2(max(1.0, float(x))))))


def shape_class(seg_row, k: int) -> str:
    """Batch shape class: mesh count, median and largest mesh rows (each
    rounded up to a power of two) and the number of eigenpairs."""
    sizes = np.diff(np.asarray(seg_row, dtype=np.int64))
    return f"k{int(k)}-meshes{_pow2(len(sizes))}-med{_pow2(np.median(sizes))}-max{_pow2(sizes.max())}"


def device_key() -> str:
    import torch

    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{p.name}-sm{p.multi_processor_count}-cc{p.major}{p.minor}"


def cache_path() -> Path:
    env = os.environ.get("LAPY_AUTOTUNE_CACHE")
    return Path(env) if env else Path.home() / ".cache" / "lapy_gb300" / "autotune.json"


class TuneCache:
    """Choices by (device, shape class), persisted as JSON."""

    def __init__(self, path: Path | str | None = None):
        self.path = Path(path) if path else cache_path()
        try:
            self.data = json.loads(self.path.read_text())
        except (OSError, ValueError):
            self.data = {}

    def get(self, device: str, shape: str) -> dict | None:
        entry = self.data.get(device, {}).get(shape)
        return dict(entry["choice"]) if entry else None

    def put(self, device: str, shape: str, choice: dict, report=None) -> None:
        self.data.setdefault(device, {})[shape] = {"choice": dict(choice), "report": report or []}
        self.path.parent.mkdir(parents=True, exist_ok=True)
        tmp = self.path.with_suffix(".tmp")
        tmp.write_text(json.dumps(self.data, indent=1, sort_keys=True))
        os.replace(tmp, self.path)


def descend(measure, start: dict | None = None, candidates: dict | None = None, margin: float = 0.03):
    """Coordinate descent: for each knob in turn, try its candidates with the
    other knobs fixed at the current choice and keep the fastest, unless it is
    less than `margin` faster than the current one.  `measure(choice)` returns
    seconds (inf for a failed run).  Returns (choice, [(choice, seconds)])."""
    cur = dict(start or DEFAULT)
    cands = candidates or CANDIDATES
    report = []
    best_t = measure(dict(cur))
    report.append((dict(cur), best_t))
    for knob, values in cands.items():
        for v in values:
            if cur.get(knob) == v:
                continue
            trial = dict(cur, **{knob: v})
            t = measure(trial)
            report.append((trial, t))
            if t < best_t * (1.0 - margin):
                cur, best_t = trial, t
    return cur, report


def stratified_sample(seg_row, size: int) -> list[int]:
    """Indices of up to `size` meshes spread over the size distribution (sorted
    by rows, evenly spaced ranks; the largest mesh always included)."""
    sizes = np.diff(np.asarray(seg_row, dtype=np.int64))
    order = np.argsort(sizes, kind="stable")
    if len(order) <= size:
        return sorted(order.tolist())
    picks = np.unique(np.round(np.linspace(0, len(order) - 1, size)).astype(int))
    return sorted(order[picks].tolist())


def solver_tuning(choice: dict) -> dict:
    """The keys of a choice that the eigensolver's tuning struct takes."""
    return {k: v for k, v in choice.items() if k in SOLVER_KEYS}


def timed_trial(fem, k: int, choice: dict, repeats: int = 1, sync=lambda: None) -> float:
    """Median seconds of `repeats` eigensolves of `fem` with the knobs of
    `choice`; inf when a solve fails or the solver rejects a knob value (such
    a choice is never kept)."""
    times = []
    for _ in range(repeats):
        sync()
        t0 = time.perf_counter()
        try:
            _, _, info = fem.eigs(k=k, block=int(choice["block"]), tuning=solver_tuning(choice))
        except ValueError:
            return float("inf")
        sync()
        if any(int(s) != 0 for s in info["status"]):
            return float("inf")
        times.append(time.perf_counter() - t0)
    return float(np.median(times))


def calibrate(meshes, k: int = 50, sample: int = 32, candidates: dict | None = None, cache: TuneCache | None = None,
              repeats: int = 1) -> tuple[dict, list]:
    """Time the candidates on a stratified sample of `meshes` and store the
    choice for their shape class.  Returns (choice, report)."""
    import torch

    from .shapedna import BatchedFEM, BatchInput

    seg = np.cumsum([0] + [len(m.v) for m in meshes])
    idx = stratified_sample(seg, sample)
    fem = BatchedFEM.from_input(BatchInput([meshes[i] for i in idx]), lump=False)
    fem.eigs(k=k, block=DEFAULT["block"], tuning=solver_tuning(DEFAULT))  # warm-up

    choice, report = descend(lambda c: timed_trial(fem, k, c, repeats, torch.cuda.synchronize),
                             candidates=candidates)
    cache = cache or TuneCache()
    cache.put(device_key(), shape_class(seg, k), choice,
              [{"choice": c, "seconds": t} for c, t in report])
    return choice, report


def choice_for(meshes_or_seg_row, k: int, cache: TuneCache | None = None) -> dict:
    """The cached choice for this batch's shape class on this device, or the
    defaults when none was calibrated."""
    if isinstance(meshes_or_seg_row, (list, tuple)) and meshes_or_seg_row and hasattr(meshes_or_seg_row[0], "v"):
        seg = np.cumsum([0] + [len(m.v) for m in meshes_or_seg_row])
    else:
        seg = np.asarray(meshes_or_seg_row)
    got = (cache or TuneCache()).get(device_key(), shape_class(seg, k))
    return dict(DEFAULT, **(got or {}))


__all__ = ["DEFAULT", "CANDIDATES", "TuneCache", "calibrate", "choice_for", "descend", "shape_class",
           "stratified_sample", "solver_tuning", "device_key", "cache_path", "timed_trial"]
