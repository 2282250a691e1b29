"""The two-level learned preconditioner (sfem_set_coarse_space): the coarse correction
P Kc^-1 P^T r of grid-cell aggregates against the FP64 oracle of oracle/coarse_oracle.py (tangent
probed from the oracle's own product at the rest state, rigid-body basis, dense Cholesky), and the
learned flexible-CG Newton solve with it: the same equilibrium (certified by the oracle's residual)
in fewer Krylov iterations.  The reference has no coarse space: parity is against the oracle."""
import os

import numpy as np
import pytest

from oracle import coarse_oracle as co
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WEIGHTS = os.path.join(ROOT, "solidfem_gb300", "data", "gnn_slab.bin")


def slab(nx, ny, nz):
    from solidfem_gb300.mesh import box_lattice, random_top_traction

    h = 1.0 / 64
    m = box_lattice(nx, ny, nz, extent=(nx * h, ny * h, nz * h), jitter=0.2, seed=0)
    return m, m.face_nodes(2, 0), random_top_traction(m, seed=10000), h


def test_coarse_correction_matches_oracle():
    from solidfem_gb300 import FemPhysicsMatrixFree

    m, fixed, f, h = slab(16, 8, 8)
    p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, young=1e5, poisson=0.49, density=1070.0, gravity=(0, 0, 0),
                             material=3, precision="fp32")
    cell = 4 * h
    p.set_coarse_space(cell)
    o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.49, 1070.0, (0, 0, 0), 3)
    X = o.free_positions().reshape(-1, 3)
    aid = co.aggregate_cells(X, cell)
    P = co.rigid_body_basis(X, aid)
    K = co.probe_tangent(o)
    Kc = co.coarse_matrix(K, P)
    rng = np.random.default_rng(4)
    for _ in range(2):
        r = rng.normal(size=3 * o.n_free)
        z_ref = P @ np.linalg.solve(Kc, P.T @ r)
        z = p.coarse_apply(r.reshape(-1, 3)).ravel()
        err = np.linalg.norm(z - z_ref) / np.linalg.norm(z_ref)
        print(f"coarse correction vs oracle ({P.shape[1]} coarse DOFs): {err:.2e}")
        # W = R Kc^-1 R^T is stored in FP16 times a power of two: each entry rounded to 2^-12 relative
        # (about 3e-4 on the correction for these sizes, measured in numpy on the same problem)
        assert err <= 1e-3


@pytest.mark.parametrize("modes", [12, 30])
def test_polynomial_coarse_correction_matches_oracle(modes):
    """The affine (12) and quadratic (30) modes per aggregate (sfem_set_coarse_space_modes) against the
    oracle's polynomial basis (orthonormalised per aggregate its own way: the same span, so the same
    correction)."""
    from solidfem_gb300 import FemPhysicsMatrixFree

    m, fixed, f, h = slab(16, 8, 8)
    p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, young=1e5, poisson=0.49, density=1070.0, gravity=(0, 0, 0),
                             material=3, precision="fp32")
    cell = 4 * h
    from solidfem_gb300 import _native as nat

    with pytest.raises(nat.SfemError):
        p.set_coarse_space(cell, modes=7)
    assert p.coarse_info()["aggregates"] == 0  # a failed set-up leaves none
    p.set_coarse_space(cell, modes=modes)
    info = p.coarse_info()
    assert info["aggregates"] > 0 and min(info["tangent_s"], info["coarse_matrix_s"], info["factorisation_s"]) >= 0
    o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.49, 1070.0, (0, 0, 0), 3)
    X = o.free_positions().reshape(-1, 3)
    aid = co.aggregate_cells(X, cell)
    P = co.poly_basis(X, aid, 1 if modes == 12 else 2)
    assert info["coarse_dofs"] == P.shape[1], (info, P.shape)
    K = co.probe_tangent(o)
    Kc = co.coarse_matrix(K, P)
    rng = np.random.default_rng(5)
    for _ in range(2):
        r = rng.normal(size=3 * o.n_free)
        z_ref = P @ np.linalg.solve(Kc, P.T @ r)
        z = p.coarse_apply(r.reshape(-1, 3)).ravel()
        err = np.linalg.norm(z - z_ref) / np.linalg.norm(z_ref)
        print(f"{modes}-mode coarse correction vs oracle ({P.shape[1]} coarse DOFs): {err:.2e}")
        assert err <= 1e-3  # W in FP16, as above


def test_two_level_learned_solve_fewer_iterations_same_equilibrium():
    from solidfem_gb300 import PC_LEARNED, FemPhysicsMatrixFree
    from solidfem_gb300.learned import LearnedPreconditioner

    m, fixed, f, h = slab(64, 16, 16)
    res = {}
    for cell, modes in ((0.0, 6), (8 * h, 6), (8 * h, 12), (8 * h, 30)):
        p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, young=1e5, poisson=0.49, density=1070.0, gravity=(0, 0, 0),
                                 material=3, precision="fp32")
        p.set_operator("assembled")
        LearnedPreconditioner(p).load(WEIGHTS)
        p.set_coarse_space(cell, modes=modes)
        p.set_nodal_loads(f)
        st = p.newton_solve(rel_tol=1e-8, max_newton=30, max_cg=100000, precond=PC_LEARNED)
        assert st["status"] == 0 and st["rel_res"] <= 1e-8, (cell, st)
        res[(cell, modes)] = (p.get_positions(), st)
        p.close()
    (x1, s1), (x2, s2), (x3, s3), (x4, s4) = res[(0.0, 6)], res[(8 * h, 6)], res[(8 * h, 12)], res[(8 * h, 30)]
    o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.49, 1070.0, (0, 0, 0), 3)
    o.set_nodal_loads(f)
    r0 = np.linalg.norm(o.gradients())
    sh = np.zeros_like(x2)
    sh[o.reshuffle_map()] = x2
    o.set_positions_shuffled(sh)
    r2 = np.linalg.norm(o.gradients()) / r0
    sh[o.reshuffle_map()] = x3
    o.set_positions_shuffled(sh)
    r3 = np.linalg.norm(o.gradients()) / r0
    sh[o.reshuffle_map()] = x4
    o.set_positions_shuffled(sh)
    r4 = np.linalg.norm(o.gradients()) / r0
    err = np.linalg.norm(x2 - x1) / np.linalg.norm(x1 - m.nodes)
    err3 = np.linalg.norm(x3 - x1) / np.linalg.norm(x1 - m.nodes)
    print(f"learned: {s1['cg_iters']} CG its in {s1['newton_iters']} Newton, {s1['seconds']:.3f} s; with the coarse "
          f"space (cells of 8h): {s2['cg_iters']} CG its in {s2['newton_iters']} Newton, {s2['seconds']:.3f} s; "
          f"affine modes: {s3['cg_iters']} CG its, {s3['seconds']:.3f} s; quadratic modes: {s4['cg_iters']} CG its, "
          f"{s4['seconds']:.3f} s; oracle |r|/|r0| {r2:.2e} / {r3:.2e} / {r4:.2e}, solutions differ by {err:.1e} / "
          f"{err3:.1e}")
    err4 = np.linalg.norm(x4 - x1) / np.linalg.norm(x1 - m.nodes)
    assert r2 <= 1.5e-8 and r3 <= 1.5e-8 and r4 <= 1.5e-8
    assert err <= 1e-6 and err3 <= 1e-6 and err4 <= 1e-6
    assert s2["cg_iters"] < 0.8 * s1["cg_iters"]
    assert s4["cg_iters"] < s3["cg_iters"] < s2["cg_iters"]
