"""N>1 path of bench.py on CPU: two gloo ranks.

The batched ShapeDNA workload shards meshes across ranks (independent units,
no data-path collective); the only collective is the max over ranks of the
timed region.  These tests run that logic with world_size 2 on the host.
"""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        meshes, lv = bench.make_batch(3, seed=bench.rank_seed(11, rank), levels=(1, 2))
        fingerprint = float(sum(np.abs(m.v).sum() for m in meshes))
        slowest = bench.max_over_ranks(1.5 + rank, world, device="cpu")
        out[rank] = (fingerprint, slowest, [len(m.v) for m in meshes])
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_ranks_shard_meshes_and_take_max_time():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    assert set(out.keys()) == {0, 1}
    (f0, s0, n0), (f1, s1, n1) = out[0], out[1]
    assert f0 != f1  # each rank builds its own meshes
    assert s0 == s1 == 2.5  # every rank reports the slowest rank's time
    assert all(n in (42, 162) for n in n0 + n1)


def test_single_rank_time_is_local():
    import bench

    assert bench.max_over_ranks(3.25, 1) == 3.25
    assert bench.rank_seed(5, 0) == 5 and bench.rank_seed(5, 1) != 5


def test_reference_arm_json_contract():
    """`bench.py --impl reference` (the SciPy method on the host cores) prints
    one JSON line with the keys the measurement contract needs."""
    import json
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    out = subprocess.run([sys.executable, str(root / "bench.py"), "--impl", "reference", "--meshes", "8",
                          "--cpu-per-level", "1", "--steps", "1", "--warmup", "0"],
                         capture_output=True, text=True, timeout=600, cwd=str(root))
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "spectra/s"
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["cpu_model"] and line["ms_per_step"] > 0
    assert line["config"]["workload"].startswith("batched ShapeDNA: 8 deformed icospheres")
