"""The coarse-space oracle (a two-level preconditioner for the flexible-CG inner solves) checked by
its algebraic properties: the probed tangent is the FP64 oracle's product, the rigid-body basis is
orthonormal and spans the rigid motions, the coarse matrix is symmetric positive definite, and the
two-level preconditioners need fewer flexible-CG iterations than the one-level ones for the same
solution (the reference has no coarse space)."""
import os

import numpy as np

from oracle import coarse_oracle as co
from oracle import gnn_oracle as go
from oracle.oracle import Oracle
from solidfem_gb300.mesh import box_lattice, random_top_traction

WEIGHTS = os.path.join(os.path.dirname(__file__), "..", "solidfem_gb300", "data", "gnn_slab.bin")


def slab(nx, ny, nz):
    """The bench workload's element size (h = 1/64), material (neo-Hookean, nu = 0.49) and load."""
    m = box_lattice(nx, ny, nz, extent=(4.0 * nx / 256, 1.0 * ny / 64, 1.0 * nz / 64), jitter=0.2, seed=0)
    fixed = m.face_nodes(2, 0)
    o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.49, 1070.0, (0, 0, 0), 3)
    f = np.zeros_like(m.nodes)
    f[o.reshuffle_map()] = random_top_traction(m, seed=7)
    o.set_nodal_loads(f)
    return o


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_probed_tangent_is_the_oracle_product():
    o = slab(8, 4, 4)
    rng = np.random.default_rng(0)
    o.set_free_positions(o.free_positions() + 1e-4 * rng.normal(size=3 * o.n_free))
    K = co.probe_tangent(o)
    for _ in range(3):
        d = rng.normal(size=3 * o.n_free)
        assert rel(K @ d, o.matvec(d)) <= 1e-12
    assert abs(K - K.T).max() <= 1e-12 * abs(K).max()


def test_rigid_body_basis_is_orthonormal_and_spans_rigid_motions():
    o = slab(8, 4, 4)
    X = o.free_positions().reshape(-1, 3)
    aid = co.aggregate_cells(X, 4 / 64)
    P = co.rigid_body_basis(X, aid)
    np.testing.assert_allclose((P.T @ P).toarray(), np.eye(P.shape[1]), atol=1e-12)
    assert P.shape[1] <= 6 * (int(aid.max()) + 1)
    for e in np.eye(3):
        for v in (np.tile(e, X.shape[0]), np.cross(e, X).ravel()):
            assert np.linalg.norm(v - P @ (P.T @ v)) <= 1e-10 * np.linalg.norm(v)
    # the compact form (offsets and one 6 x 6 matrix per aggregate) gives the same columns
    d, R = co.rigid_body_factors(X, aid)
    rng = np.random.default_rng(1)
    r = rng.normal(size=3 * X.shape[0])
    rc = np.zeros((R.shape[0], 6))  # restriction: R_a^T (sum r_i, sum d_i x r_i)
    ri = r.reshape(-1, 3)
    np.add.at(rc, aid, np.hstack([ri, np.cross(d, ri)]))
    rc = np.einsum("aij,ai->aj", R, rc)
    cols = np.cumsum([0] + [int((abs(R[a]).sum(axis=0) > 0).sum()) for a in range(R.shape[0])])
    packed = np.concatenate([rc[a, :cols[a + 1] - cols[a]] for a in range(R.shape[0])])
    np.testing.assert_allclose(packed, P.T @ r, rtol=1e-10, atol=1e-12 * np.abs(P.T @ r).max())
    y = rng.normal(size=P.shape[1])  # prolongation: u_a + omega_a x d_i, (u_a, omega_a) = R_a y_a
    ya = np.zeros((R.shape[0], 6))
    for a in range(R.shape[0]):
        ya[a, :cols[a + 1] - cols[a]] = y[cols[a]:cols[a + 1]]
    uw = np.einsum("aij,aj->ai", R, ya)
    z = uw[aid, :3] + np.cross(uw[aid, 3:], d)
    np.testing.assert_allclose(z.ravel(), P @ y, rtol=1e-10, atol=1e-12 * np.abs(P @ y).max())


def test_two_level_preconditioners_cut_iterations():
    o = slab(32, 8, 8)
    K = co.probe_tangent(o)
    b = o.gradients()
    dinv = 1.0 / K.diagonal()
    X = o.free_positions().reshape(-1, 3)
    P = co.rigid_body_basis(X, co.aggregate_cells(X, 4 / 64))
    Kc = co.coarse_matrix(K, P)
    assert abs(Kc - Kc.T).max() <= 1e-10 * abs(Kc).max()
    assert np.linalg.eigvalsh(Kc).min() > 0
    # the block form a device assembly uses gives the same matrix
    aid = co.aggregate_cells(X, 4 / 64)
    d, R = co.rigid_body_factors(X, aid)
    np.testing.assert_allclose(co.coarse_matrix_blocks(K, aid, d, R), Kc, rtol=0, atol=1e-10 * abs(Kc).max())

    params = np.fromfile(WEIGHTS, dtype=np.float32)
    Am = go.free_graph(o.tets(), o.n_bcs, o.n_nodes)

    def jacobi(r):
        return dinv * r

    def learned(r):
        return go.forward_poly(params, Am, r, dinv)

    x_j, it_j = co.fcg(K, b, jacobi)
    x_jc, it_jc = co.fcg(K, b, co.two_level(jacobi, P, Kc))
    x_l, it_l = co.fcg(K, b, learned)
    x_lc, it_lc = co.fcg(K, b, co.two_level(learned, P, Kc))
    print(f"{K.shape[0]} DOFs, coarse {Kc.shape[0]}: Jacobi {it_j}, + coarse {it_jc}; learned {it_l}, + coarse {it_lc}")
    for x in (x_jc, x_l, x_lc):
        assert rel(x, x_j) < 1e-5
    assert it_jc <= 0.35 * it_j and it_lc <= 0.85 * it_l
