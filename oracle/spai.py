"""TEST INFRASTRUCTURE ONLY -- CPU restatement of the learned factored sparse
approximate inverse (per-edge MLP) that the CUDA kernels are compared with.

No counterpart exists in the reference (lapy solves with splu); this module
states the method the CUDA kernels implement so that their features, network
outputs, factor entries, loss and gradients can be compared entry by entry.

Method.  For an SPD system K = alpha M + beta A on a mesh pattern, G is lower
triangular on the pattern's lower part (diagonal included).  For row i with
lower neighbours N_i = {j < i : K_ij != 0} the network emits w_ij per edge and

    q_i  = (e_i - w_i)' K (e_i - w_i)
         = K_ii - 2 sum_j w_ij K_ij + sum_{j,k in N_i} w_ij w_ik K_jk
    G_ii = q_i ** -0.5,   G_ij = -w_ij G_ii,

so that diag(G K G') = 1 and z = G' G r is SPD for every w (w = 0 is
Jacobi).  The training loss is the Kaporin functional of G K G',
sum_i log q_i (up to a constant), whose exact minimiser per row is the
factorised sparse approximate inverse (FSAI); its gradient is

    dL/dw_ij = (-2 K_ij + 2 sum_{k in N_i} w_ik K_jk) / q_i.

Features of edge (i, j), j < i, for K = alpha M + beta A with mean edge
length h of the mesh (segment):
    f0 = -A_ij (cotangent weight), f1 = |v_i - v_j| / h,
    f2 = m_i / h^2, f3 = m_j / h^2 (lumped vertex masses: row sums of M),
    f4 = log(t / h^2) with t = beta / alpha, f5 = sigma (0 for heat systems).
Network: 6 -> 64 -> 64 -> 1, tanh hidden activations, weights rounded to
BF16 for the forward pass (FP32 master copy), FP32 arithmetic.
"""

from __future__ import annotations

import numpy as np
from scipy import sparse

NF, H = 6, 64
LAYOUT = (("W1", (H, NF)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (1, H)), ("b3", (1,)))
NPARAM = sum(int(np.prod(s)) for _, s in LAYOUT)


def unpack(theta: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in LAYOUT:
        k = int(np.prod(shape))
        out[name] = theta[o:o + k].reshape(shape)
        o += k
    return out


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def init_params(seed: int = 0) -> np.ndarray:
    """Glorot-scaled hidden layers; a small output layer, so that w ~ 0 (Jacobi) at the start."""
    rng = np.random.default_rng(seed)
    p = []
    for name, shape in LAYOUT:
        if name.startswith("b"):
            p.append(np.zeros(shape, np.float32))
        elif name == "W3":
            p.append((rng.standard_normal(shape) * 1e-3).astype(np.float32))
        else:
            p.append((rng.standard_normal(shape) * np.sqrt(1.0 / shape[1])).astype(np.float32))
    return np.concatenate([x.ravel() for x in p]).astype(np.float32)


def lower_edges(K: sparse.csr_matrix):
    """Strictly lower entries (i, j), j < i, in row-major CSR order."""
    K = sparse.csr_matrix(K)
    K.sort_indices()
    rows = np.repeat(np.arange(K.shape[0]), np.diff(K.indptr))
    m = K.indices < rows
    return rows[m].astype(np.int64), K.indices[m].astype(np.int64)


def features(v, A, M, ei, ej, t_eff: float, sigma: float, h: float) -> np.ndarray:
    A = sparse.csr_matrix(A)
    mass = np.asarray(sparse.csr_matrix(M).sum(axis=1)).ravel()
    aij = np.asarray(A[ei, ej]).ravel()
    d = np.asarray(v, np.float64)[ei] - np.asarray(v, np.float64)[ej]
    ln = np.sqrt(np.sum(d * d, axis=1))
    f = np.empty((len(ei), NF), np.float32)
    f[:, 0] = -aij
    f[:, 1] = ln / h
    f[:, 2] = mass[ei] / h ** 2
    f[:, 3] = mass[ej] / h ** 2
    f[:, 4] = np.log(t_eff / h ** 2)
    f[:, 5] = sigma
    return f


def forward(theta: np.ndarray, f: np.ndarray, round_bf16: bool = True):
    P = {k: (bf16(x) if round_bf16 else np.asarray(x, np.float32)) for k, x in unpack(theta).items()}
    z1 = f @ P["W1"].T + P["b1"]
    h1 = np.tanh(z1)
    z2 = h1 @ P["W2"].T + P["b2"]
    h2 = np.tanh(z2)
    w = (h2 @ P["W3"].T + P["b3"])[:, 0]
    return w.astype(np.float32), (f, h1, h2, P)


def backward(cache, dw: np.ndarray) -> np.ndarray:
    """Gradient of sum_e dw_e * w_e with respect to the (FP32 master) parameters
    (straight-through the BF16 rounding)."""
    f, h1, h2, P = cache
    g = {}
    d3 = dw[:, None].astype(np.float32)                      # E x 1
    g["W3"] = d3.T @ h2
    g["b3"] = d3.sum(0)
    dz2 = (d3 @ P["W3"]) * (1.0 - h2 * h2)                   # E x H
    g["W2"] = dz2.T @ h1
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ P["W2"]) * (1.0 - h1 * h1)
    g["W1"] = dz1.T @ f
    g["b1"] = dz1.sum(0)
    return np.concatenate([g[name].ravel() for name, _ in LAYOUT]).astype(np.float64)


def factor(K: sparse.csr_matrix, ei, ej, w):
    """G (CSR, lower with diagonal), q, the loss sum_i log q_i and dL/dw."""
    K = sparse.csr_matrix(K)
    K.sort_indices()
    n = K.shape[0]
    w = np.asarray(w, np.float64)
    kd = K.diagonal()
    kij = np.asarray(K[ei, ej]).ravel()
    q = kd.copy()
    dq = -2.0 * kij
    starts = np.searchsorted(ei, np.arange(n + 1))
    for i in range(n):
        a, b = starts[i], starts[i + 1]
        if a == b:
            continue
        js = ej[a:b]
        Kjj = K[js][:, js].toarray()
        wi = w[a:b]
        q[i] += -2.0 * wi @ kij[a:b] + wi @ Kjj @ wi
        dq[a:b] += 2.0 * Kjj @ wi
    gd = 1.0 / np.sqrt(q)
    dldw = dq / q[ei]
    G = sparse.csr_matrix((np.concatenate([-w * gd[ei], gd]),
                           (np.concatenate([ei, np.arange(n)]), np.concatenate([ej, np.arange(n)]))), shape=(n, n))
    return G, q, float(np.sum(np.log(q))), dldw


def fsai_w(K: sparse.csr_matrix, ei, ej) -> np.ndarray:
    """Exact minimiser of every row's q_i: w_i = K[N,N]^-1 K[N,i]."""
    K = sparse.csr_matrix(K)
    n = K.shape[0]
    w = np.zeros(len(ei))
    starts = np.searchsorted(ei, np.arange(n + 1))
    for i in range(n):
        a, b = starts[i], starts[i + 1]
        if a == b:
            continue
        js = ej[a:b]
        w[a:b] = np.linalg.solve(K[js][:, js].toarray(), np.asarray(K[js, np.full(len(js), i)]).ravel())
    return w


def pcg_iterations(K, b, prec, rtol=1e-8, maxit=20000) -> int:
    x = np.zeros(len(b))
    r = b.copy()
    bn = np.linalg.norm(b)
    z = prec(r)
    p = z.copy()
    rz = r @ z
    for it in range(maxit):
        q = K @ p
        a = rz / (p @ q)
        x += a * p
        r -= a * q
        if np.linalg.norm(r) <= rtol * bn:
            return it + 1
        z = prec(r)
        rzn = r @ z
        p = z + rzn / rz * p
        rz = rzn
    return maxit
