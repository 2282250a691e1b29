"""Batched uneven solves (the 64-body workload): independent bodies in one handle,
per-body convergence masks; every body must match its own separate solve."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batched_bodies_match_separate_solves():
    from solidfem_gb300 import FemPhysicsMatrixFree
    from solidfem_gb300.batch import BatchedBodies, c4_specs

    specs = c4_specs(8, seed=1)
    for sp in specs:
        sp.n = min(sp.n, 24)
        sp.n -= sp.n % 4
    b = BatchedBodies(specs, precision="fp64")
    st = b.solve(rel_tol=1e-9, max_newton=100)
    assert st["status"] == 0, (st, [(s.n, s.young, s.poisson) for s in specs])
    assert (st["instance_rel_res"] <= 1e-9).all()
    for k, sp in enumerate(specs):
        m = b.meshes[k]
        x = m.nodes.copy()
        x[:, 1] += b.spacing * k  # the placement used in the batch (translation does not change the solution)
        p = FemPhysicsMatrixFree(m.tets, x, m.face_nodes(0, 0), young=sp.young, poisson=sp.poisson,
                                 density=1070.0, gravity=(0, 0, -9.81), material=3)
        s1 = p.newton_solve(rel_tol=1e-9, max_newton=100)
        assert s1["status"] == 0
        u1 = p.get_positions() - x
        ub = b.displacement(k)
        assert np.linalg.norm(ub - u1) <= 1e-6 * np.linalg.norm(u1), k


def test_c4_sixty_four_bodies_fp32_refined():
    """The full configuration: 64 bodies, n in [8, 64], one handle, FP32 Krylov with the FP64
    residual; every body reaches 1e-8 of its own initial residual."""
    from solidfem_gb300.batch import BatchedBodies, c4_specs

    specs = c4_specs(64, seed=0)
    b = BatchedBodies(specs, precision="fp32")
    t = time.time()
    st = b.solve(rel_tol=1e-8, max_newton=200)
    wall = time.time() - t
    print(f"C4: {len(specs)} bodies, {b.phys.n_tets} tets, status {st['status']}, newton {st['newton_iters']}, "
          f"cg {st['cg_iters']}, device {st['seconds']:.3f} s, wall {wall:.3f} s, "
          f"max body rel res {st['instance_rel_res'].max():.2e}")
    assert st["status"] == 0
    assert (st["instance_rel_res"] <= 1e-8).all()
