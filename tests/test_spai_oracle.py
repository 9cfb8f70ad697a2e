"""CPU checks of the learned-SPAI oracle: its gradients against finite
differences, the FSAI weights as the minimiser of the loss, and w = 0 as the
Jacobi preconditioner."""

from __future__ import annotations

import numpy as np
import pytest
from scipy import sparse

import oracle
from oracle import spai


@pytest.fixture(scope="module")
def system():
    from lapy_gb300 import meshes

    m = meshes.sh_deform(meshes.icosphere(2), seed=4)
    A, M = oracle.assemble_scipy(m.v, m.t)
    K = sparse.csr_matrix(A + 0.05 * M)
    K.sort_indices()
    ei, ej = spai.lower_edges(K)
    f = spai.features(m.v, A, M, ei, ej, 20.0, -0.05, oracle.avg_edge_length(m.v, m.t))
    return K, ei, ej, f


def test_loss_gradient_in_w(system):
    K, ei, ej, _ = system
    w = np.random.default_rng(0).uniform(-0.2, 0.2, len(ei))
    _, _, loss, dldw = spai.factor(K, ei, ej, w)
    rng = np.random.default_rng(1)
    for e in rng.choice(len(ei), 8, replace=False):
        h = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[e] += h
        wm[e] -= h
        fd = (spai.factor(K, ei, ej, wp)[2] - spai.factor(K, ei, ej, wm)[2]) / (2 * h)
        assert abs(fd - dldw[e]) <= 1e-5 * max(1.0, abs(fd))


def test_backward_matches_finite_differences(system):
    K, ei, ej, f = system
    theta = spai.init_params(3).astype(np.float64)
    theta[-65:] = np.random.default_rng(2).standard_normal(65) * 0.1  # non-trivial output layer
    dw = np.random.default_rng(5).standard_normal(len(ei)).astype(np.float32)

    def obj(th):
        w, _ = spai.forward(th.astype(np.float32), f, round_bf16=False)
        return float(np.dot(dw.astype(np.float64), w.astype(np.float64)))

    _, cache = spai.forward(theta.astype(np.float32), f, round_bf16=False)
    g = spai.backward(cache, dw)
    rng = np.random.default_rng(7)
    for p in rng.choice(spai.NPARAM, 12, replace=False):
        h = 1e-2
        tp, tm = theta.copy(), theta.copy()
        tp[p] += h
        tm[p] -= h
        fd = (obj(tp) - obj(tm)) / (2 * h)
        assert abs(fd - g[p]) <= 2e-2 * max(1.0, abs(fd)), (p, fd, g[p])


def test_fsai_minimises_the_loss(system):
    K, ei, ej, _ = system
    wf = spai.fsai_w(K, ei, ej)
    _, _, lf, dl = spai.factor(K, ei, ej, wf)
    assert np.abs(dl).max() < 1e-8
    for s in range(3):
        wn = wf + np.random.default_rng(s).normal(0, 1e-2, len(wf))
        assert spai.factor(K, ei, ej, wn)[2] > lf
    _, _, l0, _ = spai.factor(K, ei, ej, np.zeros(len(ei)))
    assert l0 > lf


def test_zero_output_is_jacobi(system):
    K, ei, ej, _ = system
    G, q, _, _ = spai.factor(K, ei, ej, np.zeros(len(ei)))
    np.testing.assert_allclose((G.T @ G).toarray(), np.diag(1.0 / K.diagonal()), rtol=1e-14, atol=0)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0], np.float32)
    r = spai.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] + 3.140625) < 1e-7 and r[4] == 0.0
