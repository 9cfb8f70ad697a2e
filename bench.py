"""Benchmark: batched ShapeDNA spectra (k=50) of deformed icospheres on one GB300.

Workload ("batched ShapeDNA"): 512 meshes, icosphere level drawn uniformly from
{3, 4, 5, 6} per mesh (642 .. 40,962 vertices), each deformed radially by
r = 1 + 0.1 sum_{l<=8,m} c_lm Y_lm with c_lm ~ N(0,1)/(1+l) from a per-mesh
seed; per mesh the k = 50 smallest eigenpairs of A x = lambda M x (cotangent
stiffness, consistent mass) by shift-invert at sigma = -0.01.

One step = assembly of the whole batch (symbolic + numeric, one block-diagonal
CSR) + the batched block shift-invert Lanczos solve, with the meshes resident
in HBM (``value``).  ``e2e`` runs the public API (``compute_shapedna_batch``)
from host arrays: mesh upload, assembly, eigensolve, eigenvalue download.

The same line carries the second half of the metric, ``heat``: heat solves/s
on the same batch (one backward-Euler step (M_s + t_s A_s) u = e_0 per mesh,
lumped mass, t_s = mean edge length squared, lapy/heat.py:114-232), resident
and end to end.  ``plain`` legs time the unbatched GPU method (one mesh at a
time through ``Solver.eigs`` / ``heat.diffusion``, Jacobi-PCG) on a stratified
sample, so that batched vs plain is measured in the same run.

``--impl reference`` times the reference's CPU method (SciPy splu + eigsh, the
oracle's restatement of lapy/solver.py) on a stratified sample of the same
meshes with all host cores.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "k=50 spectra/s (batched ShapeDNA, eig rel err <= 1e-8)"
# ncu dram__bytes_read.sum + dram__bytes_write.sum per pcg_kernel launch of the 512-mesh step
PCG_TRAFFIC_PER_LAUNCH = 9.175e12 / 147
K_EIG = 50


# ----------------------------------------------------------------------------- workload
def make_batch(n_meshes: int, seed: int, levels=(3, 4, 5, 6)):
    """Deterministic deformed icospheres (per-mesh seed), level uniform in ``levels``."""
    from lapy_gb300 import meshes

    rng = np.random.default_rng(seed)
    lv = rng.choice(levels, size=n_meshes)
    return meshes.deformed_icospheres(lv.tolist(), [seed * 100003 + i for i in range(n_meshes)]), lv


def rank_seed(seed: int, rank: int) -> int:
    """Each rank solves its own shard of meshes (independent units, no exchange)."""
    return seed + 7919 * rank


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """Slowest rank's time: the job is done when every shard is done."""
    if world <= 1:
        return x
    import torch

    tt = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
    return float(tt.item())


def stratified(lv, per_level: int):
    idx = []
    for L in sorted(set(lv.tolist())):
        idx += [i for i in range(len(lv)) if lv[i] == L][:per_level]
    return idx


def extrapolate(lv, idx, secs):
    """Whole-batch seconds from per-level mean seconds of a sample."""
    per_level_s = {}
    for i, s_ in zip(idx, secs):
        per_level_s.setdefault(int(lv[i]), []).append(s_)
    total = sum(float(np.mean(per_level_s[int(L)])) for L in lv.tolist())
    return total, {str(k): float(np.mean(v)) for k, v in per_level_s.items()}


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._thr = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._thr = threading.Thread(target=self._run, daemon=True)
        self._thr.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._thr:
            self._thr.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for s in self.samples for j in range(4) if s[4 + j].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ----------------------------------------------------------------------------- CPU baseline
def workload_name(n_meshes: int, n_vertices: int) -> str:
    """The batched workload's name; both arms print the same string."""
    return (f"batched ShapeDNA: {n_meshes} deformed icospheres (levels 3-6, {n_vertices} vertices), k=50, "
            f"sigma=-0.01, consistent mass")


def cpu_model() -> str:
    """Host CPU model (lscpu's 'Model name', else /proc/cpuinfo, else the machine)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform

    return platform.processor() or platform.machine()


def _cpu_one(args):
    """One mesh through the reference method: assembly + eigsh/splu (k
    eigenpairs), then the splu heat step.  Returns the two times and both
    results (eigenvalues, heat solution) for the accuracy check."""
    v, t, k = args
    import oracle

    t0 = time.perf_counter()
    A, M = oracle.assemble_scipy(v, t)
    ev, _ = oracle.eigs(A, M, k=k)
    t1 = time.perf_counter()
    u = oracle.diffusion(v, t, 0, m=1.0)
    return t1 - t0, time.perf_counter() - t1, np.sort(ev), u


def _run_pool(work, cores, fn=_cpu_one):
    """Run `fn` over `work` in a spawn pool, one item per worker at a time,
    BLAS threads 1; returns (results, wall seconds of the timed map)."""
    import multiprocessing as mp

    env = {"OPENBLAS_NUM_THREADS": "1", "OMP_NUM_THREADS": "1", "MKL_NUM_THREADS": "1"}
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        ctx = mp.get_context("spawn")
        with ctx.Pool(processes=min(cores, len(work))) as pool:
            pool.map(fn, work[:1])  # warm the workers' imports
            t0 = time.perf_counter()
            res = pool.map(fn, work, chunksize=1)
            wall = time.perf_counter() - t0
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return res, wall


def cpu_baseline(meshes, lv, per_level: int = 4, cores: int | None = None):
    """Reference CPU method (assembly + splu/eigsh; splu heat step) on a
    stratified sample, all cores.  Returns (spectra baseline, heat baseline,
    sample results {idx, ev, u, wall})."""
    cores = cores or len(os.sched_getaffinity(0))
    idx = stratified(lv, per_level)
    work = [(meshes[i].v, meshes[i].t, K_EIG) for i in idx]
    res, wall = _run_pool(work, cores)
    # Throughput on the whole batch: mean CPU seconds per mesh of each level
    # (measured on the sample, one mesh per worker process) times the batch's
    # level counts, spread over all cores.
    total, by_level = extrapolate(lv, idx, [r[0] for r in res])
    total_h, by_level_h = extrapolate(lv, idx, [r[1] for r in res])
    model = cpu_model()
    sample = (f"{len(work)} meshes ({per_level} per icosphere level 3-6) timed one per worker "
              f"(BLAS threads 1, sample wall {wall:.1f} s); the batch's CPU seconds "
              f"({{:.0f}}) spread over {cores} cores")
    spectra = {"value": len(meshes) / (total / cores), "unit": "spectra/s", "cores": cores, "kind": "port",
               "cpu_model": model, "sample": sample.format(total), "sec_per_mesh_by_level": by_level,
               "sample_wall_s": wall}
    heat = {"value": len(meshes) / (total_h / cores), "unit": "heat solves/s", "cores": cores, "kind": "port",
            "cpu_model": model, "sample": sample.format(total_h) + " (splu of M + t A, lumped M)",
            "sec_per_mesh_by_level": by_level_h}
    return spectra, heat, {"idx": idx, "ev": [r[2] for r in res], "u": [r[3] for r in res], "wall": wall}


def eig_accuracy(gpu_ev: np.ndarray, idx, ref_evs) -> dict:
    """GPU eigenvalues of meshes `idx` against the reference call's (eigsh in
    shift-invert mode with splu, lapy/solver.py:702-716): the largest relative
    error of lambda_1..lambda_{k-1}, and |lambda_0 - ref| / lambda_1 (lambda_0 ~ 0)."""
    rel, l0 = [], []
    for i, ref in zip(idx, ref_evs):
        g = np.asarray(gpu_ev[i], dtype=np.float64)
        lam1 = abs(ref[1])
        l0.append(abs(g[0] - ref[0]) / lam1)
        rel.append(float(np.max(np.abs(g[1:] - ref[1:]) / np.abs(ref[1:]))))
    return {"max_eig_rel_err": max(rel), "lambda0_abs_over_lambda1": max(l0), "meshes_checked": len(idx),
            "against": "scipy eigsh shift-invert + splu (the reference's call) on the host"}


def heat_accuracy(meshes, x_dev, seg_row, idx, ref_us) -> dict:
    """Batched GPU heat solutions against the reference's splu solve, in the
    lumped-mass norm: max_s ||u - u_ref||_M / ||u_ref||_M."""
    import oracle

    x = x_dev.cpu().numpy()
    errs = []
    for i, ref in zip(idx, ref_us):
        _, M = oracle.assemble_scipy(meshes[i].v, meshes[i].t, lump=True)
        w = M.diagonal()
        u = x[seg_row[i]:seg_row[i + 1]]
        errs.append(float(np.sqrt(np.sum(w * (u - ref) ** 2) / np.sum(w * ref ** 2))))
    return {"max_mnorm_rel_err": max(errs), "meshes_checked": len(idx),
            "against": "scipy splu of M + t A (the reference's call) on the host"}


# ----------------------------------------------------------------------------- GPU arm
def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_gpu(args, rank, world):
    import torch

    from lapy_gb300 import _lib, shapedna

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    meshes, lv = make_batch(args.meshes, seed=rank_seed(args.seed, rank))
    # solver knobs: calibrated for this batch's shape class on this device
    # (stratified sample, untimed) unless --block fixes the block width
    from lapy_gb300 import autotune

    tune_info = None
    if args.block:
        choice = dict(autotune.DEFAULT, block=args.block)
    else:
        t0 = time.perf_counter()
        choice, report = autotune.calibrate(meshes, k=K_EIG, sample=args.tune_sample)
        tune_info = {"sample_meshes": min(args.tune_sample, len(meshes)), "trials": len(report),
                     "calibration_s": time.perf_counter() - t0,
                     "trial_seconds": [[c, round(t, 4)] for c, t in report]}
    block = int(choice["block"])
    tuning = autotune.solver_tuning(choice)
    # inputs resident in HBM before the timed region
    batch_in = shapedna.BatchInput(meshes)
    torch.cuda.synchronize()

    def step():
        fem = shapedna.BatchedFEM.from_input(batch_in, lump=False)
        evals, _, info = fem.eigs(k=K_EIG, block=block, tuning=tuning)
        return evals, info

    for _ in range(args.warmup):
        evals, info = step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    L0 = _lib.launch_count()
    _lib.profile_reset()
    _lib.profile_enable(True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
        infos = []
        for _ in range(args.steps):
            evals, info = step()
            infos.append(info)
        ev1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    _lib.profile_enable(False)
    prof = _lib.profile_read()
    launches = _lib.launch_count() - L0
    dev_s = ev0.elapsed_time(ev1) / 1e3
    t_max = max_over_ranks(dev_s, world)
    status_ok = all(int(s) == 0 for inf in infos for s in inf["status"])

    # e2e through the public API from host buffers (mean over e2e_steps calls)
    torch.cuda.synchronize()
    e2e_steps = 0 if args.no_e2e else args.e2e_steps
    te = time.perf_counter()
    for _ in range(e2e_steps):
        res = shapedna.compute_shapedna_batch(meshes, k=K_EIG, block=block, tuning=tuning, return_vectors=False)
    torch.cuda.synchronize()
    te = time.perf_counter() - te
    h2d = sum(m.v.nbytes + m.t.size * 4 for m in meshes)
    d2h = len(meshes) * K_EIG * 8

    hbm, peak_kind = peaks()
    achieved = prof["algorithmic_bytes"] / (prof["pcg_ms"] / 1e3) / 1e9 if prof["pcg_ms"] > 0 else None
    n_total = sum(len(m.v) for m in meshes)
    line = {
        "metric": METRIC, "value": world * args.meshes * args.steps / t_max, "unit": "spectra/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 inner PCG / f64 Lanczos, Ritz and refinement", "data": "synthetic",
        "config": {"workload": workload_name(args.meshes, n_total),
                   "block": block, "tuning": choice, "autotune": tune_info, "per_gpu_meshes": args.meshes,
                   "l2": "inputs larger than L2 (batch CSR + Krylov basis >> 129 MB)",
                   "parallelism": f"replicas x{world} (meshes sharded, no collective)"},
        "e2e": ({"value": world * args.meshes * e2e_steps / te, "unit": "spectra/s", "h2d_bytes_per_step": h2d,
                 "d2h_bytes_per_step": d2h, "calls": e2e_steps} if e2e_steps else None),
        "roofline": {"bound": "hbm", "kernel": "pcg_kernel (persistent FP32 two-level PCG)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None,
                     # DRAM bytes per pcg_kernel launch, from one ncu pass over a full-size step
                     # (profiles/pcg_kernel_traffic_batched_shapedna_512.md): 1.10x the algorithmic bytes
                     "traffic": PCG_TRAFFIC_PER_LAUNCH if args.meshes == 512 else None,
                     "traffic_unit": "bytes per launch",
                     "algorithmic_per_launch": (prof["algorithmic_bytes"] / prof["pcg_launches"]
                                                if prof["pcg_launches"] else None),
                     "peak_kind": f"{peak_kind} hbm_gbs",
                     "pcg_share_of_step": prof["pcg_ms"] / 1e3 / dev_s if dev_s > 0 else None},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "status_ok": status_ok,
        "pcg": {**{k: prof[k] for k in ("pcg_launches", "pcg_iterations", "rows", "nnz")},
                "phase_ms": {k[6:-3]: prof[k] for k in prof if k.startswith("phase_")}},
        "lanczos": {"segment_steps": prof["lanczos_segment_steps"], "second_cgs_passes": prof["second_cgs_passes"]},
        "wall_s": wall,
    }
    if not args.no_spmm:
        line["spmm"] = run_spmm(batch_in, hbm, peak_kind)
    if not args.no_c1:
        line["c1"] = run_c1(args, with_cpu=rank == 0 and not args.no_cpu)
    heat_x = None
    if not args.no_heat:
        line["heat"], heat_x = run_heat(args, meshes, lv, batch_in, world)
    if not args.no_plain:
        line["plain"] = run_plain_spectra(args, meshes, lv, line["value"] / world)
    if not args.no_learned:
        line["learned"] = run_learned(args)
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"], heat_cpu, ref = cpu_baseline(meshes, lv, per_level=args.cpu_per_level)
        # accuracy of the timed step's eigenvalues on the CPU arm's sample
        line["accuracy"] = eig_accuracy(evals.cpu().numpy(), ref["idx"], ref["ev"])
        if "heat" in line:
            line["heat"]["cpu_baseline"] = heat_cpu
            line["heat"]["accuracy"] = heat_accuracy(meshes, heat_x, batch_in.seg_row, ref["idx"], ref["u"])
    return line


def _timed(fn, steps, warmup):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(steps):
        fn()
    ev1.record()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / 1e3


def run_c1(args, with_cpu, reps=5, warmup=2):
    """The single-mesh latency configuration inside the default line: icosphere
    L5 (10,242 vertices), Solver(mesh).eigs(50) from host arrays each call
    (upload, assembly, eigensolve, download), the FP64 certificate of the last
    call, and the reference method on one host core for the same mesh."""
    import torch

    from lapy_gb300 import Solver, TriaMesh, meshes

    mesh0 = meshes.icosphere(5)
    info = {}

    def call():
        fem = Solver(TriaMesh(mesh0.v.copy(), mesh0.t.copy()), lump=False)
        info["ev"], info["X"] = fem.eigs(k=50)
        info["fem"] = fem
        torch.cuda.synchronize()

    for _ in range(warmup):
        call()
    secs = []
    for _ in range(reps):
        t0 = time.perf_counter()
        call()
        secs.append(time.perf_counter() - t0)
    med = float(np.median(secs))
    out = {"workload": "icosphere L5 (10,242 vertices), Solver(mesh).eigs(50) from host arrays",
           "value": 1.0 / med, "unit": "spectra/s", "seconds_median": med, "seconds": secs,
           "certificate": eig_certificate(info["fem"], info["ev"], info["X"])}
    if with_cpu:
        cpu, ref = cpu_single("sphere-l5", mesh0, args.seed, args.cpu_timeout)
        out["cpu_baseline"] = cpu
        if ref is not None and "ev" in ref:
            out["accuracy"] = eig_accuracy(np.asarray(info["ev"])[None, :], [0], [ref["ev"]])
            out["vs_cpu_one_core"] = cpu["seconds"] / med
    return out


def run_spmm(batch_in, hbm, peak_kind, reps=20, warmup=3):
    """The pipelined FP32 SELL product alone on the headline batch's stiffness
    matrix (the PCG's SpMM outside the persistent kernel), p = 1 and 4
    columns: algorithmic bytes (value + column index per nonzero, X read once,
    Y written) over the CUDA-event time of one product."""
    import torch

    from lapy_gb300 import _device, shapedna

    fem = shapedna.BatchedFEM.from_input(batch_in, lump=False)
    sell = _device.SellF32(fem.indptr, fem.indices, fem.a_vals, fem.n, fem.nnz, seg_row=batch_in.seg_row)
    out = {"kernel": "sell_spmm_pipe_kernel (FP32 SELL, cp.async slice pipeline)", "rows": fem.n, "nnz": fem.nnz,
           "peak": hbm, "peak_kind": f"{peak_kind} hbm_gbs",
           "l2": "matrix (8 B per nonzero) >> 129 MB L2; X may stay in L2"}
    g = torch.Generator(device="cuda").manual_seed(7)

    def measure(sm, key):
        for p in (1, 4):
            x = torch.randn(fem.n, p, device="cuda", dtype=torch.float32, generator=g)
            y = torch.empty_like(x)
            for _ in range(warmup):
                sm.spmm(x, y)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(reps):
                sm.spmm(x, y)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            nbytes = fem.nnz * 8 + 2 * fem.n * p * 4
            gbs = nbytes / (ms / 1e3) / 1e9
            out[f"p{p}{key}"] = {"ms": ms, "bytes": nbytes, "achieved_gbs": gbs, "frac": gbs / hbm}

    measure(sell, "")
    del sell
    # the same matrix with every mesh's rows in reverse Cuthill-McKee order
    # (bandwidth-reducing, like the eigensolver's aggregate-contiguous order):
    # the gathers of X then stay near the rows being computed
    from scipy import sparse
    from scipy.sparse.csgraph import reverse_cuthill_mckee

    A = sparse.csr_matrix((fem.a_vals.cpu().numpy(), fem.indices.cpu().numpy(), fem.indptr.cpu().numpy()),
                          shape=(fem.n, fem.n))
    perm = np.empty(fem.n, dtype=np.int64)
    seg = batch_in.seg_row
    for i in range(len(seg) - 1):
        r0, r1 = int(seg[i]), int(seg[i + 1])
        perm[r0:r1] = r0 + reverse_cuthill_mckee(A[r0:r1, r0:r1].tocsr(), symmetric_mode=True)
    P = A[perm][:, perm].tocsr()
    P.sort_indices()
    ip = torch.from_numpy(P.indptr.astype(np.int32)).cuda()
    ix = torch.from_numpy(P.indices.astype(np.int32)).cuda()
    pv = torch.from_numpy(P.data).cuda()
    sell = _device.SellF32(ip, ix, pv, fem.n, int(P.nnz), seg_row=seg)
    measure(sell, "_rcm")
    out["rcm"] = "p*_rcm: rows of every mesh in reverse Cuthill-McKee order (scipy), same values"
    del sell, fem
    return out


def run_heat(args, meshes, lv, batch_in, world):
    """Heat solves/s: batched (resident and end to end) and plain (per mesh)."""
    import torch

    from lapy_gb300 import heat

    hb = heat.HeatBatch(batch_in, vids=0, m=1.0)
    out = {}

    def step():
        x, info = hb.solve()
        out["info"] = info
        out["x"] = x

    dev_s = max_over_ranks(_timed(step, args.steps, args.warmup), world)
    relres = float(np.max(out["info"]["relres"]))
    e2e_calls = 0 if args.no_e2e else args.e2e_steps
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(e2e_calls):
        heat.diffusion_batch(meshes, 0, m=1.0)
    torch.cuda.synchronize()
    te = time.perf_counter() - te
    # plain: the unbatched API, one mesh at a time
    idx = stratified(lv, args.plain_per_level)
    heat.diffusion(meshes[idx[0]], 0)  # warm
    secs = []
    for i in idx:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        heat.diffusion(meshes[i], 0)
        torch.cuda.synchronize()
        secs.append(time.perf_counter() - t0)
    total, by_level = extrapolate(lv, idx, secs)
    value = world * args.meshes * args.steps / dev_s
    plain = args.meshes / total
    return {"value": value, "unit": "heat solves/s", "ms_per_step": dev_s * 1e3 / args.steps,
            "max_relres": relres, "pcg_iterations": int(out["info"]["iters"]),
            "e2e": ({"value": world * args.meshes * e2e_calls / te, "unit": "heat solves/s",
                     "h2d_bytes_per_step": sum(m.v.nbytes + m.t.size * 4 for m in meshes) + 8 * len(meshes),
                     "d2h_bytes_per_step": 8 * sum(len(m.v) for m in meshes), "calls": e2e_calls}
                    if e2e_calls else None),
            "plain": {"value": world * plain, "unit": "heat solves/s",
                      "sample": f"{len(idx)} meshes ({args.plain_per_level} per level) through heat.diffusion one "
                                f"at a time, extrapolated by level counts", "sec_per_mesh_by_level": by_level},
            "vs_plain": value / (world * plain)}, out["x"]


def run_learned(args):
    """Learned SPAI: training on 4,096 level-6 systems, then Jacobi-PCG against
    learned-SPAI-PCG on held-out level-7 meshes (rel. residual 1e-8)."""
    from lapy_gb300 import spai_train

    net, hist = spai_train.train(n_meshes=128, level=6, systems=4096, batch=32, seed=args.seed)
    ev = spai_train.evaluate(net, n_test=args.learned_test, level=7, seed=args.seed + 1)
    ev4 = spai_train.evaluate(net, n_test=args.learned_test, level=7, seed=args.seed + 1, cols=4)
    return {"train": hist, "test": ev, "test_block4": ev4,
            "note": "factored SPAI G'G (per-edge MLP, BF16 weights) vs Jacobi and IC(0); same PCG, same tolerance; "
                    "test: one right-hand side per mesh, test_block4: four solved together (a Lanczos block)"}


def run_plain_spectra(args, meshes, lv, batched_per_gpu):
    """The unbatched GPU method: Solver(mesh).eigs(50) one mesh at a time."""
    import torch

    from lapy_gb300 import Solver

    idx = stratified(lv, args.plain_per_level)
    Solver(meshes[idx[0]]).eigs(k=K_EIG, precond="jacobi")  # warm
    secs = []
    for i in idx:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Solver(meshes[i]).eigs(k=K_EIG, precond="jacobi")
        torch.cuda.synchronize()
        secs.append(time.perf_counter() - t0)
    total, by_level = extrapolate(lv, idx, secs)
    plain = args.meshes / total
    return {"value": plain, "unit": "spectra/s", "per_gpu": True,
            "sample": f"{len(idx)} meshes ({args.plain_per_level} per level) through Solver(mesh).eigs(50, "
                      f"precond='jacobi') one at a time, extrapolated by level counts", "sec_per_mesh_by_level": by_level,
            "vs_plain": batched_per_gpu / plain}


# ----------------------------------------------------------------------------- single-mesh configurations
def _single_mesh(args):
    from lapy_gb300 import meshes

    if args.workload == "sphere-l5":
        return meshes.icosphere(5)
    if args.workload == "kuhn-64":
        return meshes.kuhn_cube(64, jitter=0.2, seed=args.seed)
    return meshes.deformed_icospheres([8], [args.seed])[0]


def _c2_heat_steps(fem, mesh, steps=10, t=1e-3, residuals=False):
    """u_{k+1} = (M + t A)^-1 M u_k from the centre vertex (consistent M).
    With ``residuals``, also the FP64 true residual of every step,
    ||M u_k - (M + t A) u_{k+1}|| / ||M u_k|| (computed on the device)."""
    import torch

    from lapy_gb300 import meshes
    from lapy_gb300._device import DeviceCSR, axpby, pcg_solve

    A = fem._A.as_f64()
    M = fem._M.as_f64()
    kv = M.on_pattern(A.indptr, A.indices, A.data.numel())
    axpby(t, A.data.contiguous(), 1.0, kv, out=kv)
    K = DeviceCSR(A.n, A.indptr, A.indices, kv)
    u = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    u[meshes.kuhn_center_vertex(64)] = 1.0
    res = []
    for _ in range(steps):
        b = M.matmul(u)
        u, _, _ = pcg_solve(A.indptr, A.indices, kv, A.n, kv.numel(), b, 1e-10)
        if residuals:
            res.append(float(torch.linalg.norm(b - K.matmul(u)) / torch.linalg.norm(b)))
    return (u, res) if residuals else u


def eig_certificate(fem, ev: np.ndarray, X: np.ndarray) -> dict:
    """FP64 certificate of computed eigenpairs, on the device: the largest
    relative Ritz residual ||A x - lam M x|| / (max(|lam|, lam_1) ||M x||) and
    the largest entry of X'MX - I (M-orthonormality)."""
    import torch

    A = fem._A.as_f64()
    M = fem._M.as_f64()
    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float64)).to("cuda")
    lam = torch.from_numpy(np.asarray(ev, dtype=np.float64)).to("cuda")
    AX, MX = A.matmul(Xd), M.matmul(Xd)
    R = AX - MX * lam[None, :]
    scale = torch.clamp(lam.abs(), min=abs(float(ev[1])))
    rel = torch.linalg.norm(R, dim=0) / (scale * torch.linalg.norm(MX, dim=0))
    G = Xd.T @ MX
    orth = (G - torch.eye(G.shape[0], dtype=G.dtype, device=G.device)).abs().max()
    return {"max_ritz_residual": float(rel.max()), "max_orthonormality_err": float(orth), "pairs": int(len(ev))}


def heat_certificate(mesh, u: np.ndarray, vid: int = 0, m: float = 1.0) -> dict:
    """FP64 true residual of a heat step (M + t A) u = e_vid with lumped M and
    t = m * mean edge length^2 (lapy/heat.py:204-227), on the device."""
    import torch

    from lapy_gb300 import Solver
    from lapy_gb300._device import DeviceCSR, axpby

    fem = Solver(mesh, lump=True)
    t = m * mesh.avg_edge_length() ** 2
    A = fem._A.as_f64()
    hv = fem._M.as_f64().on_pattern(A.indptr, A.indices, A.data.numel())
    axpby(t, A.data.contiguous(), 1.0, hv, out=hv)
    K = DeviceCSR(A.n, A.indptr, A.indices, hv)
    ud = torch.from_numpy(np.ascontiguousarray(u, dtype=np.float64)).to("cuda")
    b = torch.zeros_like(ud)
    b[vid] = 1.0
    return {"heat_true_relres": float(torch.linalg.norm(b - K.matmul(ud)) / torch.linalg.norm(b))}


def _cpu_single(workload, v, t, seed):
    """The reference method on one host core (oracle: SciPy splu + eigsh).
    Returns (seconds, results for the accuracy check)."""
    import oracle

    out = {}
    t0 = time.perf_counter()
    if workload == "sphere-l5":
        A, M = oracle.assemble_scipy(v, t)
        ev, _ = oracle.eigs(A, M, k=50)
        out["ev"] = np.sort(ev)
    elif workload == "kuhn-64":
        from scipy.sparse.linalg import splu

        A, M = oracle.assemble_scipy(v, t)
        out["ev"] = np.sort(oracle.eigs(A, M, k=100)[0])
        lu = splu((M + 1e-3 * A).tocsc())
        u = np.zeros(len(v))
        n = round(len(v) ** (1 / 3)) - 1
        u[n // 2 + (n + 1) * (n // 2 + (n + 1) * (n // 2))] = 1.0
        for _ in range(10):
            u = lu.solve(M @ u)
    else:
        u = oracle.diffusion(v, t, 0, m=1.0)
        out["u"] = u
        out["d"] = oracle.geodesic_f(v, t, u)
    return time.perf_counter() - t0, out


def cpu_single(workload, mesh, seed, timeout):
    import multiprocessing as mp

    os.environ.update({"OPENBLAS_NUM_THREADS": "1", "OMP_NUM_THREADS": "1"})
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        res = pool.apply_async(_cpu_single, (workload, np.asarray(mesh.v), np.asarray(mesh.t), seed))
        try:
            secs, out = res.get(timeout=timeout)
        except mp.TimeoutError:
            pool.terminate()
            return {"value": None, "unit": "runs/s", "cores": 1, "kind": "port", "cpu_model": cpu_model(),
                    "sample": f"one run of the reference method did not finish within {timeout:.0f} s"}, None
    return {"value": 1.0 / secs, "unit": "runs/s", "cores": 1, "kind": "port", "seconds": secs,
            "cpu_model": cpu_model(),
            "sample": "one full run of the reference method (SciPy splu + eigsh / splu solves), one core"}, out


def run_single(args):
    """sphere-l5 (icosphere L5, eigs 50), kuhn-64 (Kuhn 64^3 tets: eigs 100 + 10
    heat steps), sphere-l8-geodesics (deformed icosphere L8: heat + heat-method
    geodesics), from host arrays
    through the public API each step (so value and e2e coincide).  After the
    timed steps the last step's results get an FP64 certificate computed on
    the device and, where the CPU run finishes, a comparison with it."""
    import torch

    from lapy_gb300 import Solver, TetMesh, TriaMesh, diffgeo, heat

    mesh0 = _single_mesh(args)
    cls = TetMesh if args.workload == "kuhn-64" else TriaMesh
    info = {}

    def step():
        mesh = cls(mesh0.v.copy(), mesh0.t.copy())  # fresh upload every step
        if args.workload == "sphere-l5":
            fem = Solver(mesh, lump=False)
            info["ev"], info["X"] = fem.eigs(k=50)
            info["fem"] = fem
        elif args.workload == "kuhn-64":
            fem = Solver(mesh, lump=False)
            info["ev"], info["X"] = fem.eigs(k=100)
            u = _c2_heat_steps(fem, mesh)
            info["fem"] = fem
            info["u_sum"] = float(u.sum())
        else:
            u = heat.diffusion(mesh, 0, m=1.0)
            d = diffgeo.compute_geodesic_f(mesh, u)
            info["u"], info["d"] = u, d
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    with ClockSampler(torch.cuda.current_device()) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        wall = time.perf_counter() - t0
    names = {"sphere-l5": ("k=50 spectra/s (icosphere L5, 10,242 vertices)", "spectra/s"),
             "kuhn-64": ("runs/s (Kuhn 64^3 tets: eigs(100) + 10 heat steps)", "runs/s"),
             "sphere-l8-geodesics": ("runs/s (deformed icosphere L8: heat + geodesics)", "runs/s")}
    metric, unit = names[args.workload]
    v = args.steps / wall
    # FP64 certificates of the last step's results (outside the timed region)
    cert = {}
    if "ev" in info:
        cert.update(eig_certificate(info["fem"], info["ev"], info["X"]))
    if args.workload == "kuhn-64":
        _, res = _c2_heat_steps(info["fem"], None, residuals=True)
        cert["heat_max_true_relres"] = max(res)
        cert["heat_steps"] = len(res)
    if args.workload == "sphere-l8-geodesics":
        cert.update(heat_certificate(mesh0, info["u"]))
    line = {"metric": metric, "value": v, "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 inner PCG / f64 Lanczos and refinement", "data": "synthetic",
            "config": {"workload": args.workload, "vertices": int(len(mesh0.v)), "elements": int(len(mesh0.t))},
            "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": int(mesh0.v.nbytes + mesh0.t.size * 4),
                    "d2h_bytes_per_step": int(8 * (50 if args.workload == "sphere-l5" else len(mesh0.v)))},
            "clocks": clk.summary(), "certificate": cert}
    if not args.no_cpu:
        line["cpu_baseline"], ref = cpu_single(args.workload, mesh0, args.seed, args.cpu_timeout)
        acc = {}
        if ref is not None and "ev" in ref and "ev" in info:
            acc = eig_accuracy(np.asarray(info["ev"])[None, :], [0], [ref["ev"]])
        if ref is not None and "u" in ref:
            import oracle

            _, Ml = oracle.assemble_scipy(mesh0.v, mesh0.t, lump=True)
            w = Ml.diagonal()
            acc["heat_mnorm_rel_err"] = float(np.sqrt(np.sum(w * (info["u"] - ref["u"]) ** 2) /
                                                      np.sum(w * ref["u"] ** 2)))
            acc["geodesic_max_abs_diff_over_max"] = float(np.max(np.abs(info["d"] - ref["d"])) /
                                                          np.max(np.abs(ref["d"])))
            acc["against"] = "the reference method on the host (splu heat step; geodesics with its singular splu)"
        if acc:
            line["accuracy"] = acc
    return line


def run_reference(args):
    """The reference's CPU method (the oracle's restatement: SciPy splu +
    eigsh, splu heat step) on the host cores.  One step = one stratified
    sample of the batch (per_level meshes of each level), timed; the batch's
    throughput is extrapolated from the per-level CPU seconds."""
    meshes, lv = make_batch(args.meshes, seed=args.seed)
    n_total = sum(len(m.v) for m in meshes)
    for _ in range(args.warmup):
        cpu_baseline(meshes, lv, per_level=args.cpu_per_level)
    vals, heats, walls = [], [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        sp, ht, _ = cpu_baseline(meshes, lv, per_level=args.cpu_per_level)
        walls.append(time.perf_counter() - t0)
        vals.append(sp)
        heats.append(ht)
    v = statistics.median([x["value"] for x in vals])
    base = vals[0]
    hv = statistics.median([x["value"] for x in heats])
    return {"metric": METRIC, "value": v, "unit": "spectra/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(walls), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name(args.meshes, n_total),
                       "step": f"one stratified sample of {args.cpu_per_level * 4} meshes ({args.cpu_per_level} per "
                               f"level) through the CPU method, wall-timed; value extrapolates the per-level CPU "
                               f"seconds to the {args.meshes}-mesh batch over {base['cores']} cores"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "spectra/s", "cores": base["cores"], "kind": "port",
                             "cpu_model": base["cpu_model"], "sample": base["sample"]},
            "e2e": {"value": v, "unit": "spectra/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "heat": {"value": hv, "unit": "heat solves/s", "cpu_baseline": heats[0]}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="shapedna", choices=["shapedna", "sphere-l5", "kuhn-64", "sphere-l8-geodesics"],
                    help="shapedna: the batched headline (512 meshes); the others: single-mesh workloads")
    ap.add_argument("--meshes", type=int, default=512)
    ap.add_argument("--block", type=int, default=0, help="Lanczos block width; 0: autotuned with the other knobs")
    ap.add_argument("--tune-sample", type=int, default=32, help="meshes of the autotuner's calibration sample")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-per-level", type=int, default=4)
    ap.add_argument("--plain-per-level", type=int, default=1)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-timeout", type=float, default=600.0, help="single-mesh workloads: CPU run time limit (s)")
    ap.add_argument("--no-heat", action="store_true")
    ap.add_argument("--no-spmm", action="store_true", help="skip the standalone SELL SpMM leg")
    ap.add_argument("--no-c1", action="store_true", help="skip the single-mesh (icosphere L5) leg")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--learned-test", type=int, default=32, help="held-out level-7 meshes of the learned-SPAI leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the public-API end-to-end leg (profiling runs)")
    ap.add_argument("--e2e-steps", type=int, default=3, help="public-API calls averaged by the e2e legs")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    if args.workload != "shapedna":
        if rank == 0:
            print(json.dumps(run_single(args)), flush=True)
        return
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    line = run_gpu(args, rank, world)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
