"""Learned factorised sparse approximate inverse (per-edge MLP) for the PCG.

No counterpart exists in the reference, which factorises its systems with
``splu`` (lapy/solver.py:707, lapy/heat.py:223); this is the preconditioner
option of the GPU solves.  For an SPD system ``K = alpha M + beta A`` on a
mesh pattern a per-edge network emits the off-diagonal ratios ``w_ij`` of a
lower-triangular factor ``G``; every row is normalised exactly
(``q_i = (e_i - w_i)' K (e_i - w_i)``, ``G_ii = q_i^-1/2``,
``G_ij = -w_ij G_ii``) so ``G'G`` is SPD for every network output and zero
output is Jacobi.  The network (6 -> 64 -> 64 -> 1, tanh, BF16 weights, FP32
arithmetic) is trained on the GPU by the library's own forward, backward and
Adam kernels to minimise ``sum_i log q_i``, the Kaporin functional of
``G K G'`` (whose exact per-row minimiser is FSAI).

Edge features (per lower entry (i, j), mean edge length h of the mesh):
``-A_ij`` (cotangent weight), ``|v_i - v_j| / h``, ``m_i / h^2``,
``m_j / h^2`` (lumped masses), ``log(t / h^2)`` with ``t = beta / alpha``
and ``sigma`` (0 for heat systems).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from . import _lib
from ._device import dptr, stream, workspace

NF, HID = 6, 64
_LAYOUT = (("W1", (HID, NF)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)), ("W3", (1, HID)), ("b3", (1,)))
NPARAM = sum(int(np.prod(s)) for _, s in _LAYOUT)
WEIGHTS_FILE = Path(__file__).resolve().parent / "data" / "spai_weights.npz"


def init_params(seed: int = 0) -> np.ndarray:
    """Scaled-normal hidden layers, zero biases and a small output layer (w ~ 0:
    training starts from Jacobi)."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in _LAYOUT:
        if name.startswith("b"):
            parts.append(np.zeros(shape, np.float32))
        elif name == "W3":
            parts.append((rng.standard_normal(shape) * 1e-3).astype(np.float32))
        else:
            parts.append((rng.standard_normal(shape) * np.sqrt(1.0 / shape[1])).astype(np.float32))
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


@dataclass
class SpaiPattern:
    """Lower / upper split of a symmetric CSR pattern with a full diagonal."""

    n: int
    nnz: int
    lptr: torch.Tensor
    lcol: torch.Tensor
    lpos: torch.Tensor
    uptr: torch.Tensor
    ucol: torch.Tensor
    umap: torch.Tensor

    @property
    def nlower(self) -> int:
        return (self.nnz + self.n) // 2

    @classmethod
    def build(cls, indptr: torch.Tensor, indices: torch.Tensor, n: int, nnz: int) -> "SpaiPattern":
        L = _lib.lib()
        m = (nnz + n) // 2
        i32 = dict(dtype=torch.int32, device="cuda")
        lptr, uptr = torch.empty(n + 1, **i32), torch.empty(n + 1, **i32)
        lcol, lpos, ucol, umap = (torch.empty(m, **i32) for _ in range(4))
        ws = workspace(L.lapy_spai_pattern_workspace_bytes(n))
        _lib.check(L.lapy_spai_pattern(n, dptr(indptr), dptr(indices), nnz, dptr(lptr), dptr(lcol), dptr(lpos),
                                       dptr(uptr), dptr(ucol), dptr(umap), dptr(ws), ws.numel(), stream()),
                   "spai_pattern")
        return cls(n, nnz, lptr, lcol, lpos, uptr, ucol, umap)


class SpaiNet:
    """Network parameters on the device: FP32 master copy, BF16 forward copy,
    Adam moments."""

    def __init__(self, theta: np.ndarray | None = None, seed: int = 0):
        L = _lib.lib()
        if L.lapy_spai_param_count() != NPARAM:
            raise RuntimeError("spai: parameter layout of the library differs")
        theta = init_params(seed) if theta is None else np.asarray(theta, np.float32).ravel()
        if theta.size != NPARAM:
            raise ValueError(f"spai: expected {NPARAM} parameters, got {theta.size}")
        self.theta = torch.from_numpy(theta.copy()).to("cuda")
        self.wb = torch.empty(NPARAM, dtype=torch.bfloat16, device="cuda")
        self.m = torch.zeros(NPARAM, dtype=torch.float32, device="cuda")
        self.v = torch.zeros(NPARAM, dtype=torch.float32, device="cuda")
        self.grad = torch.zeros(NPARAM, dtype=torch.float32, device="cuda")
        self.step = 0
        _lib.check(L.lapy_spai_weights_to_bf16(NPARAM, dptr(self.theta), dptr(self.wb), stream()), "spai_to_bf16")

    @classmethod
    def load(cls, path: str | Path = WEIGHTS_FILE) -> "SpaiNet":
        with np.load(path) as d:
            return cls(d["theta"])

    def save(self, path: str | Path, **meta) -> None:
        Path(path).parent.mkdir(parents=True, exist_ok=True)
        np.savez(path, theta=self.theta.cpu().numpy(), **{k: np.asarray(v) for k, v in meta.items()})

    def forward(self, feat: torch.Tensor) -> torch.Tensor:
        ne = feat.shape[0]
        w = torch.empty(ne, dtype=torch.float32, device="cuda")
        _lib.check(_lib.lib().lapy_spai_forward(ne, dptr(feat), dptr(self.wb), dptr(w), stream()), "spai_forward")
        return w

    def backward(self, feat: torch.Tensor, dldw: torch.Tensor, scale: float) -> torch.Tensor:
        L = _lib.lib()
        ne = feat.shape[0]
        ws = workspace(L.lapy_spai_backward_workspace_bytes(ne))
        _lib.check(L.lapy_spai_backward(ne, dptr(feat), dptr(self.wb), dptr(dldw), scale, dptr(self.grad), dptr(ws),
                                        ws.numel(), stream()), "spai_backward")
        return self.grad

    def adam(self, lr: float = 3e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        self.step += 1
        _lib.check(_lib.lib().lapy_spai_adam(NPARAM, dptr(self.theta), dptr(self.grad), dptr(self.m), dptr(self.v),
                                             dptr(self.wb), lr, beta1, beta2, eps, self.step, stream()),
                   "spai_adam")


class SpaiSystems:
    """A batch of SPD systems K_s = alpha_s M_s + beta_s A_s on one device
    batch of meshes (block-diagonal CSR), with their edge features.

    ``kind`` 'heat': K = M (lumped) + t_s A; 'shift': K = A - sigma M
    (consistent mass), the shift-invert operator of the eigensolver."""

    def __init__(self, batch_input, kind: str, t=None, sigma: float = -0.01):
        from .shapedna import BatchedFEM

        if kind not in ("heat", "shift"):
            raise ValueError("kind must be 'heat' or 'shift'")
        L = _lib.lib()
        self.input = batch_input
        nseg = len(batch_input.seg_row) - 1
        fem = BatchedFEM.from_input(batch_input, lump=(kind == "heat"))
        self.fem = fem
        self.n, self.nnz, self.nseg = fem.n, fem.nnz, nseg
        self.indptr, self.indices = fem.indptr, fem.indices
        seg = batch_input.seg_row_dev
        f64 = dict(dtype=torch.float64, device="cuda")
        self.h = torch.empty(nseg, **f64)
        _lib.check(L.lapy_seg_avg_edge_length(dptr(batch_input.mesh.v), batch_input.mesh.coords_f32, nseg, dptr(seg),
                                              dptr(fem.indptr), dptr(fem.indices), 1.0, dptr(self.h), None, stream()),
                   "seg_avg_edge_length")
        k = torch.empty(fem.nnz, **f64)
        if kind == "heat":
            if isinstance(t, torch.Tensor):
                self.t = t.to(device="cuda", dtype=torch.float64).contiguous()
            else:
                tt = np.broadcast_to(np.asarray(1e-3 if t is None else t, np.float64), (nseg,)).copy()
                self.t = torch.from_numpy(tt).to("cuda")
            self.sigma = torch.zeros(nseg, **f64)
            ones = torch.ones(nseg, **f64)
            _lib.check(L.lapy_csr_seg_axpby(nseg, dptr(seg), dptr(fem.indptr), dptr(fem.pattern.diag_pos),
                                            dptr(self.t), dptr(fem.a_vals), dptr(ones), dptr(fem.m_vals), 1, dptr(k),
                                            stream()), "csr_seg_axpby")
        else:
            self.t = torch.full((nseg,), -1.0 / sigma, **f64)
            self.sigma = torch.full((nseg,), sigma, **f64)
            _lib.check(L.lapy_vec_axpby(fem.nnz, 1.0, dptr(fem.a_vals), -sigma, dptr(fem.m_vals), dptr(k), stream()),
                       "vec_axpby")
        self.k = k
        self.pattern = SpaiPattern.build(fem.indptr, fem.indices, fem.n, fem.nnz)
        self.feat = torch.empty(self.pattern.nlower, NF, dtype=torch.float32, device="cuda")
        mass = torch.empty(fem.n, **f64)
        p = self.pattern
        _lib.check(L.lapy_spai_features(fem.n, nseg, dptr(seg), dptr(batch_input.mesh.v), batch_input.mesh.coords_f32,
                                        dptr(fem.indptr), dptr(fem.a_vals), dptr(fem.m_vals), int(kind == "heat"),
                                        dptr(p.lptr), dptr(p.lcol), dptr(p.lpos), dptr(self.t), dptr(self.sigma),
                                        dptr(self.h), dptr(mass), dptr(self.feat), stream()), "spai_features")

    def factor(self, w: torch.Tensor, grad: bool = False):
        """(G on the lower pattern, G' on the upper pattern, log q per row,
        dL/dw or None)."""
        L = _lib.lib()
        p = self.pattern
        g = torch.empty(p.nlower, dtype=torch.float32, device="cuda")
        logq = torch.empty(self.n, dtype=torch.float64, device="cuda")
        dldw = torch.empty(p.nlower, dtype=torch.float32, device="cuda") if grad else None
        _lib.check(L.lapy_spai_factor(self.n, dptr(self.indptr), dptr(self.indices), dptr(self.k), dptr(p.lptr),
                                      dptr(p.lcol), dptr(p.lpos), dptr(w), dptr(g), dptr(logq), dptr(dldw),
                                      stream()), "spai_factor")
        gt = torch.empty_like(g)
        _lib.check(L.lapy_spai_transpose_values(p.nlower, dptr(p.umap), dptr(g), dptr(gt), stream()),
                   "spai_transpose_values")
        return g, gt, logq, dldw

    def solve(self, B: torch.Tensor, g=None, gt=None, rtol: float = 1e-8, maxiter: int = 20000, ic0: bool = False):
        """PCG on every segment: the learned factor (g, gt), IC(0) (ic0=True)
        or Jacobi (neither).  Returns (X, relres per (segment, column), PCG
        iterations)."""
        from ._device import ic0_pcg_solve, pcg_solve

        if ic0:
            x, relres, iters, _ = ic0_pcg_solve(self.indptr, self.indices, self.k, self.n, self.nnz, B, rtol, maxiter,
                                                seg_row=self.input.seg_row)
            return x, relres, iters
        if g is None:
            return pcg_solve(self.indptr, self.indices, self.k, self.n, self.nnz, B, rtol, maxiter,
                             seg_row=self.input.seg_row)
        L = _lib.lib()
        p = self.pattern
        squeeze = B.dim() == 1
        Bm = B.reshape(self.n, -1).contiguous()
        ncol = Bm.shape[1]
        seg = np.ascontiguousarray(self.input.seg_row, dtype=np.int32)
        X = torch.empty_like(Bm)
        ws = workspace(L.lapy_spai_pcg_workspace_bytes(self.n, self.nnz, self.nseg, seg.ctypes.data, ncol))
        status = np.zeros(self.nseg * ncol, np.int32)
        relres = np.zeros(self.nseg * ncol, np.float64)
        iters = C.c_int64(0)
        _lib.check(L.lapy_spai_pcg_solve(self.n, dptr(self.indptr), dptr(self.indices), dptr(self.k), self.nnz,
                                         self.nseg, seg.ctypes.data, ncol, dptr(Bm), dptr(X), rtol, maxiter, 1e-4,
                                         dptr(p.lptr), dptr(p.lcol), dptr(g), dptr(p.uptr), dptr(p.ucol), dptr(gt),
                                         status.ctypes.data, relres.ctypes.data, C.byref(iters), dptr(ws), ws.numel(),
                                         stream()), "spai_pcg_solve")
        bad = status[status != 0]
        if bad.size:
            _lib.check(int(bad[0]), "spai_pcg_solve")
        return (X[:, 0] if squeeze else X), relres, int(iters.value)


_DEFAULT_NET: SpaiNet | None = None


def default_net() -> SpaiNet:
    """The shipped network (trained by lapy_gb300.spai_train), loaded once."""
    global _DEFAULT_NET
    if _DEFAULT_NET is None:
        _DEFAULT_NET = SpaiNet.load(WEIGHTS_FILE)
    return _DEFAULT_NET


def learned_solve(sys_: SpaiSystems, B: torch.Tensor, rtol: float, maxiter: int = 20000, net: SpaiNet | None = None):
    """Factor with the network and solve (X, relres, iterations)."""
    net = net or default_net()
    g, gt, _, _ = sys_.factor(net.forward(sys_.feat))
    return sys_.solve(B, g, gt, rtol=rtol, maxiter=maxiter)


def train_step(net: SpaiNet, sys_: SpaiSystems, lr: float = 3e-3) -> float:
    """One Adam step on the mean Kaporin loss of a batch; returns the loss
    before the step (mean log q over the batch's rows)."""
    w = net.forward(sys_.feat)
    _, _, logq, dldw = sys_.factor(w, grad=True)
    net.backward(sys_.feat, dldw, 1.0 / sys_.n)
    net.adam(lr)
    return float(logq.mean())


def kaporin_loss(net: SpaiNet | None, sys_: SpaiSystems) -> float:
    """Mean log q of the factor (net None: Jacobi, w = 0)."""
    w = net.forward(sys_.feat) if net is not None else torch.zeros(sys_.pattern.nlower, dtype=torch.float32,
                                                                   device="cuda")
    return float(sys_.factor(w)[2].mean())


__all__ = ["SpaiNet", "SpaiPattern", "SpaiSystems", "train_step", "kaporin_loss", "init_params", "NPARAM",
           "default_net", "learned_solve"]
