"""Training and held-out evaluation of the learned SPAI preconditioner.

Workload: systems (M + t A) x = b (lumped M, t log-uniform in [1e-4, 1e-1])
and (A - sigma M) x = b (consistent M, sigma = -0.01) on deformed level-6
icospheres (radius 1 + 0.1 sum_{l<=8} c_lm Y_lm, c_lm ~ N(0,1)/(1+l)), trained
in batches of meshes (one block-diagonal system per step, half of the steps
heat systems, half shift-invert systems); evaluated on held-out deformed
level-7 icospheres against Jacobi-PCG at relative residual 1e-8, b ~ N(0,1).

    python -m lapy_gb300.spai_train --out lapy_gb300/data/spai_weights.npz
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import meshes
from .shapedna import BatchInput
from .spai import SpaiNet, SpaiSystems, kaporin_loss, train_step


def _sync_time() -> float:
    torch.cuda.synchronize()
    return time.perf_counter()


def train(n_meshes: int = 128, level: int = 6, systems: int = 4096, batch: int = 32, lr: float = 3e-3,
          seed: int = 0, log=None):
    """Train a fresh network; returns (net, history dict)."""
    rng = np.random.default_rng(seed)
    ms = meshes.deformed_icospheres([level] * n_meshes, [10_000 + seed * 1_000_003 + i for i in range(n_meshes)])
    groups = [BatchInput(ms[g:g + batch]) for g in range(0, n_meshes, batch)]
    net = SpaiNet(seed=seed)
    steps = max(1, systems // batch)
    losses = []
    t0 = _sync_time()
    for step in range(steps):
        inp = groups[step % len(groups)]
        nseg = len(inp.seg_row) - 1
        if step % 2 == 0:
            sysg = SpaiSystems(inp, "heat", t=10 ** rng.uniform(-4, -1, nseg))
        else:
            sysg = SpaiSystems(inp, "shift")
        losses.append(train_step(net, sysg, lr))
        if log and (step + 1) % max(1, steps // 8) == 0:
            log(f"spai train step {step + 1}/{steps}: mean log q {losses[-1]:.5f}")
    t_train = _sync_time() - t0
    return net, {"steps": steps, "systems": steps * batch, "batch": batch, "meshes": n_meshes, "level": level,
                 "train_s": t_train, "loss_first": losses[0], "loss_last": losses[-1]}


def evaluate(net: SpaiNet, n_test: int = 16, level: int = 7, seed: int = 1, rtol: float = 1e-8,
             batch: int = 64, cols: int = 1) -> dict:
    """Jacobi-PCG, IC(0)-PCG and learned-SPAI-PCG on held-out meshes, same
    right-hand sides and tolerance; the meshes are solved in block-diagonal
    batches of `batch` (times summed over batches, iteration counts and
    residuals the largest over batches).  `cols` right-hand-side columns per
    mesh are solved together (one pass over the matrix and the factors serves
    all of them, as for a Lanczos block)."""
    rng = np.random.default_rng(seed)
    ms = meshes.deformed_icospheres([level] * n_test, [50_000 + seed * 1_000_003 + i for i in range(n_test)])
    out = {"meshes": n_test, "level": level, "rows": 0, "rtol": rtol, "batch": batch, "cols": cols}
    acc = {}
    for g0 in range(0, n_test, batch):
        inp = BatchInput(ms[g0:g0 + batch])
        out["rows"] += int(inp.seg_row[-1])
        nb = len(inp.seg_row) - 1
        for kind in ("heat", "shift"):
            t = 10 ** rng.uniform(-4, -1, nb) if kind == "heat" else None
            sysg = SpaiSystems(inp, kind, t=t)
            shape = (sysg.n,) if cols == 1 else (sysg.n, cols)
            b = torch.from_numpy(rng.standard_normal(shape)).to("cuda")
            sysg.solve(b, rtol=rtol)  # warm
            t0 = _sync_time()
            _, rj, itj = sysg.solve(b, rtol=rtol)
            tj = _sync_time() - t0
            t0 = _sync_time()
            g, gt, _, _ = sysg.factor(net.forward(sysg.feat))
            tf = _sync_time() - t0
            t0 = _sync_time()
            _, rl, itl = sysg.solve(b, g, gt, rtol=rtol)
            tl = _sync_time() - t0
            sysg.solve(b, rtol=rtol, ic0=True)  # warm
            t0 = _sync_time()
            _, ri, iti = sysg.solve(b, rtol=rtol, ic0=True)  # factorization included
            ti = _sync_time() - t0
            a = acc.setdefault(kind, {"jacobi_iters": 0, "learned_iters": 0, "ic0_iters": 0, "jacobi_solve_s": 0.0,
                                      "learned_setup_s": 0.0, "learned_solve_s": 0.0, "ic0_solve_s_incl_factor": 0.0,
                                      "max_relres_jacobi": 0.0, "max_relres_learned": 0.0, "max_relres_ic0": 0.0,
                                      "kaporin_jacobi": [], "kaporin_learned": []})
            a["jacobi_iters"] = max(a["jacobi_iters"], itj)
            a["learned_iters"] = max(a["learned_iters"], itl)
            a["ic0_iters"] = max(a["ic0_iters"], iti)
            a["jacobi_solve_s"] += tj
            a["learned_setup_s"] += tf
            a["learned_solve_s"] += tl
            a["ic0_solve_s_incl_factor"] += ti
            a["max_relres_jacobi"] = max(a["max_relres_jacobi"], float(np.max(rj)))
            a["max_relres_learned"] = max(a["max_relres_learned"], float(np.max(rl)))
            a["max_relres_ic0"] = max(a["max_relres_ic0"], float(np.max(ri)))
            a["kaporin_jacobi"].append(kaporin_loss(None, sysg))
            a["kaporin_learned"].append(kaporin_loss(net, sysg))
            del sysg, g, gt
            torch.cuda.empty_cache()
    for kind, a in acc.items():
        a["kaporin_jacobi"] = float(np.mean(a["kaporin_jacobi"]))
        a["kaporin_learned"] = float(np.mean(a["kaporin_learned"]))
        a["iters_ratio"] = a["learned_iters"] / max(a["jacobi_iters"], 1)
        out[kind] = a
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=None)
    ap.add_argument("--meshes", type=int, default=128)
    ap.add_argument("--systems", type=int, default=4096)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--test", type=int, default=16)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()
    net, hist = train(args.meshes, 6, args.systems, args.batch, seed=args.seed, log=print)
    ev = evaluate(net, args.test)
    if args.out:
        net.save(args.out, steps=hist["steps"], systems=hist["systems"], loss_last=hist["loss_last"])
    print(json.dumps({"train": hist, "eval": ev}), flush=True)


if __name__ == "__main__":
    main()
