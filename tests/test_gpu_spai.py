"""Learned SPAI on the GPU against the CPU oracle (oracle/spai.py): pattern
split, edge features, network forward (BF16 weights), factor / loss / dL/dw,
the parameter gradient, and what training buys over Jacobi-PCG on held-out
meshes (assessed by iterations, true residual and the FP64 solution)."""

from __future__ import annotations

import numpy as np
import pytest
from scipy import sparse
from scipy.sparse.linalg import spsolve

import oracle
from oracle import spai as ospai

pytestmark = pytest.mark.gpu


def _meshes(levels_seeds):
    from lapy_gb300 import meshes

    return [meshes.sh_deform(meshes.icosphere(lv), seed=s) for lv, s in levels_seeds]


def _oracle_system(mesh, kind, t):
    A, M = oracle.assemble_scipy(mesh.v, mesh.t, lump=(kind == "heat"))
    if kind == "heat":
        K, teff, sig = M + t * A, t, 0.0
    else:
        K, teff, sig = A + 0.01 * M, 100.0, -0.01
    K = sparse.csr_matrix(K)
    K.sort_indices()
    ei, ej = ospai.lower_edges(K)
    f = ospai.features(mesh.v, A, M, ei, ej, teff, sig, oracle.avg_edge_length(mesh.v, mesh.t))
    return K, ei, ej, f


@pytest.fixture(scope="module")
def batch(cuda_ok):
    from lapy_gb300.shapedna import BatchInput

    ms = _meshes([(2, 11), (3, 12), (2, 13)])
    return ms, BatchInput(ms)


@pytest.mark.parametrize("kind", ["shift", "heat"])
def test_pattern_features_forward_factor_backward(batch, kind):
    import torch

    from lapy_gb300.spai import SpaiNet, SpaiSystems

    ms, inp = batch
    t = [3e-3, 1e-2, 4e-2]
    sysg = SpaiSystems(inp, kind, t=t)
    refs = [_oracle_system(m, kind, tt) for m, tt in zip(ms, t)]
    seg = inp.seg_row
    # pattern: lower entries (incl. the diagonal) of every segment in CSR order
    lptr = sysg.pattern.lptr.cpu().numpy()
    lcol = sysg.pattern.lcol.cpu().numpy()
    off = 0
    for s, (K, ei, ej, f) in enumerate(refs):
        Kl = sparse.tril(K).tocsr()
        Kl.sort_indices()
        n0 = seg[s]
        np.testing.assert_array_equal(lptr[n0:seg[s + 1] + 1] - lptr[n0], Kl.indptr)
        np.testing.assert_array_equal(lcol[lptr[n0]:lptr[seg[s + 1]]] - n0, Kl.indices)
    ut = sysg.pattern.umap.cpu().numpy()
    assert np.all(ut >= 0) and len(np.unique(ut)) == len(ut)

    # features and forward on the strictly lower entries
    feat = sysg.feat.cpu().numpy()
    strict = np.ones(sysg.pattern.nlower, bool)
    strict[lptr[1:] - 1] = False  # diagonal slots
    fr = np.concatenate([f for (_, _, _, f) in refs])
    np.testing.assert_allclose(feat[strict], fr, rtol=2e-6, atol=2e-6)

    theta = ospai.init_params(5)
    theta[-65:] = np.random.default_rng(9).standard_normal(65).astype(np.float32) * 0.05
    net = SpaiNet(theta)
    w = net.forward(sysg.feat)
    wr, cache = ospai.forward(theta, fr)
    wg = w.cpu().numpy()[strict]
    np.testing.assert_allclose(wg, wr, rtol=0, atol=2e-5 * max(1.0, np.abs(wr).max()))

    # factor, loss and dL/dw with the same w
    g, gt, logq, dldw = sysg.factor(w, grad=True)
    wsplit = np.split(wg.astype(np.float64), np.cumsum([len(r[1]) for r in refs])[:-1])
    gl = g.cpu().numpy()
    dl = dldw.cpu().numpy()
    lq = logq.cpu().numpy()
    o = 0
    for s, ((K, ei, ej, f), ws) in enumerate(zip(refs, wsplit)):
        G, q, loss, dref = ospai.factor(K, ei, ej, ws)
        n0, n1 = seg[s], seg[s + 1]
        np.testing.assert_allclose(lq[n0:n1], np.log(q), rtol=0, atol=1e-9)
        Gd = sparse.csr_matrix((gl[lptr[n0]:lptr[n1]], lcol[lptr[n0]:lptr[n1]] - n0, lptr[n0:n1 + 1] - lptr[n0]),
                               shape=(n1 - n0, n1 - n0))
        np.testing.assert_allclose(Gd.toarray(), G.toarray(), rtol=2e-6, atol=1e-7 * np.abs(G.data).max())
        dsl = dl[lptr[n0]:lptr[n1]][strict[lptr[n0]:lptr[n1]]]
        np.testing.assert_allclose(dsl, dref, rtol=1e-4, atol=1e-6 * np.abs(dref).max())
        o += len(ei)
    # transposed factor values: G' on the upper pattern
    uptr = sysg.pattern.uptr.cpu().numpy()
    ucol = sysg.pattern.ucol.cpu().numpy()
    n = sysg.n
    Gfull = sparse.csr_matrix((gl, lcol, lptr), shape=(n, n))
    GT = sparse.csr_matrix((gt.cpu().numpy(), ucol, uptr), shape=(n, n))
    assert abs(GT - Gfull.T).max() == 0

    # parameter gradient of sum_e dL/dw_e w_e (straight through BF16)
    grad = net.backward(sysg.feat, dldw, 1.0).cpu().numpy()
    gref = ospai.backward(cache, np.concatenate([dl[lptr[seg[s]]:lptr[seg[s + 1]]][strict[lptr[seg[s]]:lptr[seg[s + 1]]]]
                                                 for s in range(len(refs))]))
    np.testing.assert_allclose(grad, gref, rtol=0, atol=2e-4 * np.abs(gref).max())
    torch.cuda.synchronize()


def test_training_beats_jacobi_on_held_out_meshes(cuda_ok):
    import torch

    from lapy_gb300.shapedna import BatchInput
    from lapy_gb300.spai import SpaiNet, SpaiSystems, kaporin_loss, train_step

    rng = np.random.default_rng(0)
    train_in = BatchInput(_meshes([(3, 100 + i) for i in range(6)]))
    systems = [SpaiSystems(train_in, "shift")] + [
        SpaiSystems(train_in, "heat", t=10 ** rng.uniform(-4, -1, 6)) for _ in range(3)]
    net = SpaiNet(seed=0)
    l0 = kaporin_loss(None, systems[0])
    for step in range(240):
        train_step(net, systems[step % len(systems)], lr=3e-3)
    assert kaporin_loss(net, systems[0]) < l0

    test_mesh = _meshes([(4, 777)])
    test_in = BatchInput(test_mesh)
    for kind, t in (("shift", None), ("heat", 1e-2)):
        sysg = SpaiSystems(test_in, kind, t=t)
        n = sysg.n
        b = torch.from_numpy(np.random.default_rng(3).standard_normal(n)).to("cuda")
        xj, rj, itj = sysg.solve(b, rtol=1e-8)
        g, gt, _, _ = sysg.factor(net.forward(sysg.feat))
        xl, rl, itl = sysg.solve(b, g, gt, rtol=1e-8)
        K, *_ = _oracle_system(test_mesh[0], kind, t)
        xref = spsolve(sparse.csc_matrix(K), b.cpu().numpy())
        for x, r in ((xj, rj), (xl, rl)):
            assert np.all(r <= 1e-8)
            xx = x.cpu().numpy()
            assert np.linalg.norm(xx - xref) <= 1e-6 * np.linalg.norm(xref)
        if kind == "shift":
            assert itl <= 0.8 * itj, (itl, itj)
        else:
            assert itl <= itj, (itl, itj)


def test_learned_heat_matches_oracle(cuda_ok):
    """heat.diffusion / diffusion_batch with the shipped network: the FP64
    solution of the reference's system, at the heat bar (M-norm rel <= 1e-8)."""
    from lapy_gb300 import heat

    ms = _meshes([(3, 21), (4, 22)])
    vids = [0, 5]
    batch = heat.diffusion_batch(ms, vids, m=1.0, precond="learned")
    for mesh, v, ub in zip(ms, vids, batch):
        ref = oracle.diffusion(mesh.v, mesh.t, v, m=1.0)
        md = oracle.assemble_scipy(mesh.v, mesh.t, lump=True)[1].diagonal()
        u = heat.diffusion(mesh, v, m=1.0, precond="learned")
        for x in (u, ub):
            assert np.sqrt(np.sum(md * (x - ref) ** 2) / np.sum(md * ref ** 2)) <= 1e-8
    with pytest.raises(ValueError, match="precond"):
        heat.diffusion(ms[0], 0, precond="ilu")
