"""Solver front ends and failure detection on the GPU: the pysolidfem-compatible
NonlinearFEM, the nonlinear CG minimiser, quasi-static load stepping, and the error
statuses (non-finite input, inverted elements, iteration caps) -- all raised on the
host from a status the library returns; nothing here faults or traps the GPU."""
import numpy as np
import pytest

from tests.conftest import load_golden

pytestmark = pytest.mark.gpu


def test_nonlinearfem_drop_in_matches_reference_static_solve():
    from solidfem_gb300 import NonlinearFEM

    g = load_golden("box2_nh.npz")
    # the reference's PyNonlinearFEM keys; gravity defaults to -9.8 along y as in the reference
    sim = NonlinearFEM(g["tets"], g["nodes"], g["fixed"],
                       {"young": 66000.0, "poisson": 0.45, "density": 1070.0, "maxiter": 100, "tol": 1e-9})
    sim.step()
    x = sim.get_nodes()
    u, uref = x - g["nodes"], g["eq_positions"] - g["nodes"]
    assert np.linalg.norm(u - uref) <= 1e-6 * np.linalg.norm(uref)
    sim.compute_force_param_grads()
    assert sim.get_force_mu_grad().size == 3 * (g["nodes"].shape[0] - len(g["fixed"]))
    assert sim.get_shear_modulus() == pytest.approx(66000.0 / 2.9)


def test_nonlinear_cg_reaches_newton_equilibrium():
    from solidfem_gb300 import FemPhysicsMatrixFree
    from solidfem_gb300.mesh import box_lattice, lumped_face_load

    m = box_lattice(8, 2, 2, extent=(2.0, 0.5, 0.5))
    f = lumped_face_load(m, 0, 1, (0.0, 0.0, -200.0))
    kw = dict(young=1e6, poisson=0.3, density=0.0, gravity=(0, 0, 0), material=3)
    a = FemPhysicsMatrixFree(m.tets, m.nodes, m.face_nodes(0, 0), **kw)
    a.set_nodal_loads(f)
    st = a.newton_solve(rel_tol=1e-11)
    assert st["status"] == 0
    b = FemPhysicsMatrixFree(m.tets, m.nodes, m.face_nodes(0, 0), **kw)
    b.set_nodal_loads(f)
    _, r0 = b.ComputeGradients(return_norm=True)
    # NonlinearConjugateGradientMinimizer stops once |r|^2 <= eps^2 |r0|^2 with eps = 1e-2
    # (Include/NonlinearCG.h:103-107): a 1% residual, by the reference's design
    its = b.nonlinear_cg(outer_iters=20000, inner_iters=10, abs_tol=1e-7 * r0)
    _, r1 = b.ComputeGradients(return_norm=True)
    assert r1 <= 1.01e-2 * r0, (its, r1 / r0)
    ua, ub = a.get_positions() - m.nodes, b.get_positions() - m.nodes
    assert np.linalg.norm(ua - ub) <= 5e-2 * np.linalg.norm(ua)


def test_load_stepping_reaches_the_same_equilibrium():
    from solidfem_gb300 import FemPhysicsMatrixFree

    g = load_golden("c1_newton_ls.npz")
    p = FemPhysicsMatrixFree(g["tets"], g["nodes"], g["fixed"], young=1e5, poisson=0.45, density=1070.0,
                             gravity=(0.0, 0.0, -9.81), material=3)
    st = p.newton_solve(rel_tol=1e-10, max_newton=300, load_steps=5)
    assert st["status"] == 0, st
    u, uref = p.get_positions() - g["nodes"], g["eq_positions"] - g["nodes"]
    assert np.linalg.norm(u - uref) <= 1e-6 * np.linalg.norm(uref)


def _small():
    from solidfem_gb300 import FemPhysicsMatrixFree
    from solidfem_gb300.mesh import box_lattice

    m = box_lattice(6, 2, 2, extent=(1.5, 0.5, 0.5))
    return m, FemPhysicsMatrixFree(m.tets, m.nodes, m.face_nodes(0, 0), young=1e5, poisson=0.45,
                                   gravity=(0.0, 0.0, -9.81), material=3)


def test_nonfinite_input_reports_nan_status():
    from solidfem_gb300 import SfemError

    m, p = _small()
    x = m.nodes.copy()
    x[-1, 2] = np.nan
    p.set_positions(x)
    r, nrm = p.ComputeGradients(return_norm=True)
    assert not np.isfinite(nrm)
    with pytest.raises(SfemError) as ei:
        p.newton_solve(rel_tol=1e-8)
    assert ei.value.code == -3


def test_inverted_element_is_detected():
    m, p = _small()
    assert not p.CheckForInversion()
    x = m.nodes.copy()
    t = m.tets[10]
    x[t[0]] = x[t[1]] + 2.0 * (x[t[1]] - x[t[0]])  # push corner 0 through the opposite side
    p.set_positions(x)
    assert p.count_inverted() >= 1 and p.CheckForInversion()


def test_iteration_caps_report_not_converged():
    m, p = _small()
    st = p.newton_solve(rel_tol=1e-12, max_newton=1)
    assert st["status"] == 1 and st["newton_iters"] == 1
    b = np.ones((p.n_free, 3))
    x, pst = p.pcg(b, rel_tol=1e-12, max_iters=3)
    assert pst["status"] == 1 and pst["iters"] == 3


def test_solves_are_bitwise_deterministic():
    m, p = _small()
    p.newton_solve(rel_tol=1e-10)
    x1 = p.get_positions()
    p.set_positions(m.nodes)
    p.newton_solve(rel_tol=1e-10)
    np.testing.assert_array_equal(x1, p.get_positions())
