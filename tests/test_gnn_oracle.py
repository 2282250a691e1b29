"""The FP64 oracle of the learned preconditioner is pinned by central finite differences
of its own loss, and M(r) is checked to be a symmetric positive definite linear operator
(the reference has no learned component)."""
import numpy as np
import pytest

from oracle import gnn_oracle as go
from oracle.oracle import Oracle
from solidfem_gb300.mesh import box_lattice


def small_problem():
    m = box_lattice(6, 3, 3, extent=(1.5, 0.75, 0.75))
    fixed = m.face_nodes(2, 0)
    o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, (0, 0, 0), 3)
    Am = go.free_graph(o.tets(), o.n_bcs, o.n_nodes)
    dinv = 1.0 / o.jacobi_diagonal()
    return o, Am, dinv


def test_graph_is_symmetric_mean_aggregation():
    o, Am, _ = small_problem()
    A = (Am > 0).astype(float)
    assert abs(A - A.T).max() == 0
    np.testing.assert_allclose(np.asarray(Am.sum(axis=1)).ravel(), 1.0)


def test_preconditioner_is_linear_symmetric_positive_definite():
    o, Am, dinv = small_problem()
    rng = np.random.default_rng(3)
    p = rng.normal(size=go.NPARAM) * 0.1
    n = 3 * o.n_free
    u, v = rng.normal(size=(2, n))
    Mu, Mv = go.forward(p, Am, u, dinv), go.forward(p, Am, v, dinv)
    np.testing.assert_allclose(go.forward(p, Am, 2.0 * u - 3.0 * v, dinv), 2.0 * Mu - 3.0 * Mv, rtol=1e-10,
                               atol=1e-12 * np.abs(Mu).max())
    assert abs(u @ Mv - v @ Mu) <= 1e-10 * abs(u @ Mv)
    # M = D^-1/2 (c I + S^T S) D^-1/2 >= c D^-1
    c = np.exp(p[go.OFF_C])
    for w in rng.normal(size=(8, n)):
        assert w @ go.forward(p, Am, w, dinv) >= c * (w @ (dinv * w)) * (1 - 1e-12)


@pytest.mark.parametrize("mode", ["energy", "residual"])
def test_oracle_gradient_matches_central_differences(mode):
    o, Am, dinv = small_problem()
    rng = np.random.default_rng(0)
    p = rng.normal(size=go.NPARAM) * 0.1
    r = rng.normal(size=3 * o.n_free)
    e, _, _ = o.pcg(r, diag=1.0 / dinv, tol=1e-12, max_iters=20000)  # a consistent pair: K e = r
    K = o.matvec
    L, g = go.loss_grad(p, Am, r, dinv, e, K, bf16_layers=False, mode=mode)
    idx = np.concatenate([rng.choice(go.NPARAM - 1, size=40, replace=False), [go.OFF_C]])
    for k in idx:
        h = 1e-5
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (go.loss_grad(pp, Am, r, dinv, e, K, bf16_layers=False, mode=mode)[0]
              - go.loss_grad(pm, Am, r, dinv, e, K, bf16_layers=False, mode=mode)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * np.abs(g).max() + 1e-4 * abs(fd), (k, fd, g[k])


def test_folded_polynomial_equals_the_network():
    o, Am, dinv = small_problem()
    rng = np.random.default_rng(5)
    p = rng.normal(size=go.NPARAM) * 0.1
    r = rng.normal(size=3 * o.n_free)
    a, b = go.forward(p, Am, r, dinv), go.forward_poly(p, Am, r, dinv)
    assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(a)
    G, _ = go.poly_coefficients(p)
    for k in range(go.NL + 1):  # G_kj = T_k T_j^T: G_kj = G_jk^T
        for j in range(go.NL + 1):
            np.testing.assert_allclose(G[k, j], G[j, k].T, rtol=1e-12, atol=1e-14 * np.abs(G).max())
