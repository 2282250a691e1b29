"""The FP64 oracle of the learned preconditioner is pinned by central finite
differences of its own loss (the reference has no learned component)."""
import numpy as np

from oracle import gnn_oracle as go
from oracle.oracle import Oracle
from solidfem_gb300.mesh import box_lattice


def small_problem():
    m = box_lattice(6, 3, 3, extent=(1.5, 0.75, 0.75))
    fixed = m.face_nodes(2, 0)
    o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, (0, 0, 0), 3)
    Am, fnb = go.free_graph(o.tets(), o.n_bcs, o.n_nodes)
    dinv = 1.0 / o.jacobi_diagonal()
    return o, Am, fnb, dinv


def test_graph_is_symmetric_mean_aggregation():
    o, Am, fnb, _ = small_problem()
    A = (Am > 0).astype(float)
    assert abs(A - A.T).max() == 0
    np.testing.assert_allclose(np.asarray(Am.sum(axis=1)).ravel(), 1.0)
    assert fnb.any() and not fnb.all()


import pytest


@pytest.mark.parametrize("mode", ["energy", "residual"])
def test_oracle_gradient_matches_central_differences(mode):
    o, Am, fnb, dinv = small_problem()
    rng = np.random.default_rng(0)
    p = rng.normal(size=go.NPARAM) * 0.1
    r = rng.normal(size=3 * o.n_free)
    e, _, _ = o.pcg(r, diag=1.0 / dinv, tol=1e-12, max_iters=20000)  # a consistent pair: K e = r
    K = o.matvec
    L, g = go.loss_grad(p, Am, fnb, r, dinv, e, K, bf16_layers=False, mode=mode)
    idx = rng.choice(go.NPARAM, size=40, replace=False)
    for k in idx:
        h = 1e-5
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (go.loss_grad(pp, Am, fnb, r, dinv, e, K, bf16_layers=False, mode=mode)[0]
              - go.loss_grad(pm, Am, fnb, r, dinv, e, K, bf16_layers=False, mode=mode)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * np.abs(g).max() + 1e-4 * abs(fd), (k, fd, g[k])
