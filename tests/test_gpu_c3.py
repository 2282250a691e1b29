"""The headline workload's physics on a 3.1M-tet slab of the same shape and element size: box
[0,2]x[0,1]x[0,1] as 128x64x64 hexes x 6 tets (545,025 nodes / 3,145,728 tets), interior nodes
jittered U(-0.2h, 0.2h), compressible neo-Hookean E = 1e5 Pa, nu = 0.49, bottom face clamped,
smoothed random top traction N(0, 200 Pa) (load seed 10000).

The solve the bench times -- learned-preconditioner flexible CG in FP32 through the assembled
operator, FP64 Newton residual, to |r|/|r0| <= 1e-8 -- is certified by the oracle's own FP64
residual (ComputeGradients semantics, FemPhysicsMatrixFree.cpp:536-560) at the GPU's equilibrium,
and its displacement is compared with an FP64 Jacobi-PCG solve of the same load to 1e-10 (itself
certified by the oracle).  No CPU solve at this size: the residual is a size-independent check."""
import os

import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _shuffled(o, x):
    out = np.zeros_like(x)
    out[o.reshuffle_map()] = x
    return out


def test_c3_slab_fp32_learned_vs_oracle_and_fp64():
    from solidfem_gb300 import PC_JACOBI, PC_LEARNED, FemPhysicsMatrixFree
    from solidfem_gb300.learned import LearnedPreconditioner
    from solidfem_gb300.mesh import box_lattice, random_top_traction

    m = box_lattice(128, 64, 64, extent=(2.0, 1.0, 1.0), jitter=0.2, seed=0)
    assert m.n_tets == 3145728
    fixed = m.face_nodes(2, 0)
    f = random_top_traction(m, seed=10000)
    kw = dict(young=1e5, poisson=0.49, density=1070.0, gravity=(0, 0, 0), material=3)

    p32 = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, precision="fp32", **kw)
    p32.set_operator("assembled")
    LearnedPreconditioner(p32).load(os.path.join(ROOT, "solidfem_gb300", "data", "gnn_slab.bin"))
    p32.set_nodal_loads(f)
    st32 = p32.newton_solve(rel_tol=1e-8, max_newton=30, max_cg=200000, precond=PC_LEARNED)
    assert st32["status"] == 0 and st32["rel_res"] <= 1e-8, st32
    u32 = p32.get_positions() - m.nodes
    p32.close()

    p64 = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, precision="fp64", **kw)
    p64.set_operator("assembled")
    p64.set_nodal_loads(f)
    st64 = p64.newton_solve(rel_tol=1e-10, max_newton=30, max_cg=400000, precond=PC_JACOBI)
    assert st64["status"] == 0, st64
    u64 = p64.get_positions() - m.nodes
    p64.close()

    o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.49, 1070.0, (0, 0, 0), 3)
    o.set_nodal_loads(f)
    r0 = np.linalg.norm(o.gradients())
    o.set_positions_shuffled(_shuffled(o, m.nodes + u32))
    r32 = np.linalg.norm(o.gradients()) / r0
    x64 = _shuffled(o, m.nodes + u64)
    o.set_positions_shuffled(x64)
    r64 = np.linalg.norm(o.gradients()) / r0
    # the oracle evaluates positions, not displacements: rounding a position to FP64 alone moves the
    # residual by about this much (the same positions moved by one ulp at random)
    rng = np.random.default_rng(1)
    xp = x64.copy()
    xp[o.n_bcs:] = np.nextafter(xp[o.n_bcs:], np.where(rng.random(xp[o.n_bcs:].shape) < 0.5, -np.inf, np.inf))
    o.set_positions_shuffled(xp)
    floor = np.linalg.norm(o.gradients()) / r0
    err = np.linalg.norm(u32 - u64) / np.linalg.norm(u64)
    print(f"C3 slab 3.1M tets: FP32 learned {st32['seconds']:.3f} s ({st32['newton_iters']} Newton, "
          f"{st32['cg_iters']} CG), oracle |r|/|r0| {r32:.2e}; FP64 Jacobi {st64['seconds']:.2f} s "
          f"({st64['newton_iters']} Newton, {st64['cg_iters']} CG), oracle |r|/|r0| {r64:.2e} (1-ulp "
          f"position floor {floor:.2e}); displacement error FP32 vs FP64 {err:.2e}")
    # the oracle's residual agrees with the GPU's FP64 residual up to summation order
    assert r32 <= 1.5e-8
    # below 1e-9 the oracle's measure reaches the floor set by FP64 positions
    assert r64 <= max(1.5e-10, 2.0 * floor)
    # the FP32-refined solution's error against the FP64 solution (stated; bounded here)
    assert err <= 1e-5
