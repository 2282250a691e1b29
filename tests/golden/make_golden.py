"""Generate the golden fixtures in tests/golden/ from the REFERENCE's own code.

The reference's hot-path sources are compiled unmodified into
oracle/_ref/libsfem_ref.so (oracle/Makefile.ref) and driven through
oracle/ref_harness.cpp.  This script needs the reference tree
(SFEM_REF_TREE, default /root/reference) and is run in the development container only:

    python tests/golden/make_golden.py

Fixtures (npz):
  box2_nh.npz        reference model Models/box2.tet (tet1 loader swaps y<->z,
                     Source/FemIO.cpp:548), nodes 0-8 fixed as in Models/cantilever.xml,
                     neo-Hookean E=66000 nu=0.45 rho=1070 g=-9.8 (y): element-level outputs
                     and the reference's own static solve (Step(0) -> SolveNewtonLS).
  lattice_<mat>.npz  jittered 6x2x2 lattice, each material: outputs at perturbed positions.
  c1_newton_ls.npz   16x4x4 cantilever (425 nodes / 1536 tets), neo-Hookean E=1e5 nu=0.45,
                     gravity -9.81 z, x=0 clamped: the reference's SolveNewtonLS equilibrium.
  c2s_<mat>.npz      8x2x2 box [0,8]x[0,2]x[0,2] (reduced C2), E=1e6 nu=0.4, 500 Pa -z traction
                     on x=8, x=0 clamped: equilibrium from reference assembly + Eigen SparseLU.
  dyn_nh.npz         8x2x2 cantilever [0,2]x[0,0.5]x[0,0.5], neo-Hookean E=1e5 nu=0.45 rho=1070,
                     gravity -9.81 z, x=0 clamped, from rest: the reference's own Step(dt):
                     ST_EXPLICIT (dt 0.01, 10 substeps) x 3 and ST_IMPLICIT with SolveNewtonLS
                     (dt 0.01, 1 substep) x 3 -> positions and velocities after each step.

  tangent_<mat>.npz  jittered 4x2x2 lattice at perturbed positions, each material: the reference's
                     assembled tangent ElasticEnergy::AssembleStiffnessMatrix (dense, free DOFs).
  variant_<m>.npz    the same lattice for the other MaterialModelType values m = 4..12: stress,
                     gradients, energy, tangent diagonal and assembled tangent from the reference.

  nlcg_c1.npz        the C1 cantilever: the reference's NonlinearConjugateGradientMinimizer iterate after
                     k outer iterations (10 inner), for E = 1e7 (k = 1, 3, 10) and E = 1e5 (k = 1, 3).
  bw_c1.npz          the C1 cantilever: the reference's NewtonSolverBackTrack with the Bonet-Wood condition,
                     every line-search trial (Newton iteration, step length, residual norm) and the solution.

    python tests/golden/make_golden.py [--only dyn|tangent|variant|solvers]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import REF_TREE, RefHarness  # noqa: E402
from solidfem_gb300.mesh import box_lattice, lumped_face_load  # noqa: E402

REF = REF_TREE
MATS = {0: "linear", 1: "stvk", 2: "corot", 3: "nh"}


def load_tet1(path):
    """Reader for SolidFEM's 'tet1' text format (v x y z / t i j k l), y<->z swapped as
    IO::LoadFromTet1File does (Source/FemIO.cpp:506-581)."""
    nodes, tets = [], []
    with open(path) as f:
        for line in f:
            p = line.split()
            if not p:
                continue
            if p[0] == "v":
                x, y, z = map(float, p[1:4])
                nodes.append((x, z, y))
            elif p[0] == "t":
                tets.append(tuple(int(v) for v in p[1:5]))
    return np.array(nodes), np.array(tets, dtype=np.int32)


def element_outputs(ref, rng, perturb):
    x = ref.positions_shuffled().copy()
    x0 = x.copy()
    x[ref.n_bcs:] += perturb * rng.normal(size=x[ref.n_bcs:].shape)
    ref.set_positions_shuffled(x)
    d = rng.normal(size=3 * ref.n_free)
    out = dict(pos_shuffled=x, d=d, grad=ref.gradients(), matvec=ref.matvec(d), diag=ref.jacobi_diagonal(),
               stress=ref.element_stress(), energy=np.array(ref.elastic_energy()), map=ref.reshuffle_map(),
               tets_shuffled=ref.tets())
    gmu, gl, grho = ref.force_param_grads()
    out.update(gmu=gmu, glambda=gl, grho=grho)
    ref.set_positions_shuffled(x0)
    out["grad_rest"] = ref.gradients()
    return out


def dynamics():
    m = box_lattice(8, 2, 2, extent=(2.0, 0.5, 0.5))
    fixed = m.face_nodes(0, 0)
    out = dict(nodes=m.nodes, tets=m.tets, fixed=fixed, young=1e5, poisson=0.45, density=1070.0,
               gravity=np.array([0.0, 0.0, -9.81]), material=3, dt=0.01, explicit_substeps=10, steps=3)
    ref = RefHarness(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, -9.81, True, 3)
    ref.set_sim(2, 10)  # ST_EXPLICIT, mNumSteps
    xs, vs = [], []
    for _ in range(3):
        ref.step_dt(0.01)
        xs.append(ref.positions())
        vs.append(ref.velocities_shuffled()[ref.reshuffle_map()])
    out.update(explicit_positions=np.array(xs), explicit_velocities=np.array(vs))
    ref = RefHarness(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, -9.81, True, 3, solver=1, outer_iters=100,
                     abs_tol=1e-11)
    ref.set_sim(3, 1)  # ST_IMPLICIT, SolveNewtonLS per step
    xs, vs = [], []
    for _ in range(3):
        ref.step_dt(0.01)
        xs.append(ref.positions())
        vs.append(ref.velocities_shuffled()[ref.reshuffle_map()])
    out.update(implicit_positions=np.array(xs), implicit_velocities=np.array(vs))
    np.savez_compressed(os.path.join(HERE, "dyn_nh.npz"), **out)
    print("dyn: implicit tip after 3 steps", xs[-1][m.node_index(8, 2, 2)])


def tangents():
    m = box_lattice(4, 2, 2, extent=(1.0, 0.5, 0.5), jitter=0.15, seed=5)
    fixed = m.face_nodes(0, 0)
    for mat, name in MATS.items():
        ref = RefHarness(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, -9.81, True, mat)
        rng = np.random.default_rng(20 + mat)
        x = ref.positions_shuffled() + rng.normal(size=(m.n_nodes, 3)) * 0.01
        x[:ref.n_bcs] = ref.positions_shuffled()[:ref.n_bcs]
        ref.set_positions_shuffled(x.ravel())
        K = ref.assemble_dense()
        np.savez_compressed(os.path.join(HERE, f"tangent_{name}.npz"), nodes=m.nodes, tets=m.tets, fixed=fixed,
                            young=1e5, poisson=0.45, density=1070.0, material=mat, pos_shuffled=x,
                            map=ref.reshuffle_map(), K=K)
        print(f"tangent {name}: {K.shape}, |K| = {np.abs(K).max():.3e}, asym {np.abs(K - K.T).max():.2e}")


def variants():
    m = box_lattice(4, 2, 2, extent=(1.0, 0.5, 0.5), jitter=0.15, seed=5)
    fixed = m.face_nodes(0, 0)
    for mat in range(4, 13):
        ref = RefHarness(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, -9.81, True, mat)
        ref.set_force_fraction(1.0)
        rng = np.random.default_rng(40 + mat)
        x = ref.positions_shuffled() + rng.normal(size=(m.n_nodes, 3)) * 0.01
        x[:ref.n_bcs] = ref.positions_shuffled()[:ref.n_bcs]
        ref.set_positions_shuffled(x.ravel())
        np.savez_compressed(os.path.join(HERE, f"variant_{mat}.npz"), nodes=m.nodes, tets=m.tets, fixed=fixed,
                            young=1e5, poisson=0.45, density=1070.0, gravity=np.array([0.0, 0.0, -9.81]),
                            material=mat, pos_shuffled=x, map=ref.reshuffle_map(), stress=ref.element_stress(),
                            grad=ref.gradients(), energy=ref.elastic_energy(), diag=ref.jacobi_diagonal(),
                            K=ref.assemble_dense())
        print(f"variant {mat}: |grad| {np.linalg.norm(ref.gradients()):.3e} energy {ref.elastic_energy():.3e}")


def reference_solvers():
    """The reference's own nonlinear solvers on the C1 cantilever (16x4x4, gravity, x=0 clamped):
    NonlinearConjugateGradientMinimizer (Include/NonlinearCG.h:51-114, through Step(0) with
    NST_NONLINEAR_CG) after k outer iterations, and NewtonSolverBackTrack with its Bonet-Wood
    condition (SolveNewtonLS's set-up) with every line-search trial recorded."""
    m = box_lattice(16, 4, 4, extent=(4.0, 1.0, 1.0))
    fixed = m.face_nodes(0, 0)
    out = dict(nodes=m.nodes, tets=m.tets, fixed=fixed, poisson=0.45, density=1070.0,
               gravity=np.array([0.0, 0.0, -9.81]), material=3, inner_iters=10, abs_tol=1e-12)
    cases = [(1e7, 1), (1e7, 3), (1e7, 10), (1e5, 1), (1e5, 3)]
    pos = []
    for young, k in cases:
        ref = RefHarness(m.nodes, m.tets, fixed, young, 0.45, 1070.0, -9.81, True, 3, solver=3, outer_iters=k,
                         inner_iters=10, abs_tol=1e-12)
        ref.set_force_fraction(0.0)  # Step(0) of ST_STATIC solves only while mForceFraction == 0
        ref.step()
        pos.append(ref.positions())
        print(f"nlcg E={young:g} k={k}: max |u| {np.abs(pos[-1] - m.nodes).max():.4e}")
    out.update(young=np.array([c[0] for c in cases]), outer_iters=np.array([c[1] for c in cases]),
               positions=np.array(pos))
    np.savez_compressed(os.path.join(HERE, "nlcg_c1.npz"), **out)

    ref = RefHarness(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, -9.81, True, 3, solver=1, outer_iters=400,
                     abs_tol=1e-9)
    tr = ref.newton_ls_trace(400, 1e-9)
    np.savez_compressed(os.path.join(HERE, "bw_c1.npz"), nodes=m.nodes, tets=m.tets, fixed=fixed, young=1e5,
                        poisson=0.45, density=1070.0, gravity=np.array([0.0, 0.0, -9.81]), material=3,
                        abs_tol=1e-9, trial_iter=tr["it"], trial_step=tr["step"], trial_res=tr["res"], r0=tr["r0"],
                        converged=tr["converged"], eq_positions=ref.positions())
    print(f"bonet-wood: {tr['it'].max() + 1} Newton iterations, {tr['it'].size} trials, converged {tr['converged']}")


def main():
    if "--only" in sys.argv:
        {"dyn": dynamics, "tangent": tangents, "variant": variants,
         "solvers": reference_solvers}[sys.argv[sys.argv.index("--only") + 1]]()
        return
    if not os.path.isdir(REF):
        sys.exit("reference tree not present; fixtures are generated in the development container")
    rng = np.random.default_rng(20261203)

    # --- box2 fixture of the reference ---
    nodes, tets = load_tet1(os.path.join(REF, "Models", "box2.tet"))
    fixed = np.arange(9, dtype=np.int32)
    ref = RefHarness(nodes, tets, fixed, 66000.0, 0.45, 1070.0, -9.8, False, 3, solver=1, outer_iters=100,
                     abs_tol=1e-9)
    ref.set_force_fraction(1.0)
    out = element_outputs(ref, rng, 0.002)
    ref.set_force_fraction(0.0)  # Step(0) of ST_STATIC solves only while mForceFraction == 0
    ref.step()  # the reference's own Step(0): ST_STATIC -> Solve -> SolveNewtonLS
    out.update(nodes=nodes, tets=tets, fixed=fixed, young=66000.0, poisson=0.45, density=1070.0,
               gravity=np.array([0.0, -9.8, 0.0]), material=3, eq_positions=ref.positions(),
               eq_grad=ref.gradients())
    np.savez_compressed(os.path.join(HERE, "box2_nh.npz"), **out)
    print("box2: |r_eq| =", np.linalg.norm(out["eq_grad"]))

    # --- all materials on a jittered lattice ---
    m = box_lattice(6, 2, 2, extent=(1.5, 0.5, 0.5), jitter=0.2, seed=7)
    fixed = m.face_nodes(0, 0)
    for mat, name in MATS.items():
        ref = RefHarness(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, -9.81, True, mat)
        ref.set_force_fraction(1.0)
        fl = lumped_face_load(m, 0, 1, (0.0, 100.0, -300.0))
        ref.set_nodal_loads(fl)
        out = element_outputs(ref, rng, 0.01)
        out.update(nodes=m.nodes, tets=m.tets, fixed=fixed, young=1e5, poisson=0.45, density=1070.0,
                   gravity=np.array([0.0, 0.0, -9.81]), material=mat, loads=fl)
        np.savez_compressed(os.path.join(HERE, f"lattice_{name}.npz"), **out)

    # --- C1: the reference's SolveNewtonLS equilibrium ---
    m = box_lattice(16, 4, 4, extent=(4.0, 1.0, 1.0))
    fixed = m.face_nodes(0, 0)
    ref = RefHarness(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, -9.81, True, 3, solver=1, outer_iters=400,
                     abs_tol=1e-9)
    ref.set_force_fraction(1.0)
    r0 = np.linalg.norm(ref.gradients())
    ref.set_force_fraction(0.0)
    ref.step()
    g = ref.gradients()
    np.savez_compressed(os.path.join(HERE, "c1_newton_ls.npz"), nodes=m.nodes, tets=m.tets, fixed=fixed,
                        young=1e5, poisson=0.45, density=1070.0, gravity=np.array([0.0, 0.0, -9.81]), material=3,
                        eq_positions=ref.positions(), r0=r0, r_eq=np.linalg.norm(g))
    print("c1: |r0| =", r0, " |r_eq| =", np.linalg.norm(g), " tip:", ref.positions()[m.node_index(16, 4, 4)])

    # --- reduced C2: dead traction, corotational and neo-Hookean, direct Newton ---
    m = box_lattice(8, 2, 2, extent=(8.0, 2.0, 2.0))
    fixed = m.face_nodes(0, 0)
    fl = lumped_face_load(m, 0, 1, (0.0, 0.0, -500.0))
    for mat in (2, 3):
        ref = RefHarness(m.nodes, m.tets, fixed, 1e6, 0.4, 1070.0, 0.0, True, mat)
        ref.set_nodal_loads(fl)
        ref.set_force_fraction(1.0)
        r0 = np.linalg.norm(ref.gradients())
        # corotational: the reference's analytic tangent is inconsistent with its force, so the
        # harness Newton uses the reference's finite-difference Jacobian scheme instead
        its, rn = (ref.newton_fd if mat == 2 else ref.newton_direct)(max_iters=200, rel_tol=1e-13)
        np.savez_compressed(os.path.join(HERE, f"c2s_{MATS[mat]}.npz"), nodes=m.nodes, tets=m.tets, fixed=fixed,
                            young=1e6, poisson=0.4, density=1070.0, gravity=np.zeros(3), material=mat, loads=fl,
                            eq_positions=ref.positions(), r0=r0, r_eq=rn, newton_iters=its)
        print(f"c2s {MATS[mat]}: its={its} |r0|={r0:.3e} |r|={rn:.3e}")
    dynamics()
    tangents()
    variants()
    reference_solvers()


if __name__ == "__main__":
    main()
