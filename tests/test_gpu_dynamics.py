"""Dynamics on the GPU (FemPhysicsMatrixFree with mTimeStep != 0, Step with ST_EXPLICIT /
ST_IMPLICIT): the backward-Euler residual, tangent product and Jacobi diagonal against the
oracle (bit-identical to the reference's own code, tests/test_oracle_pin.py), and whole steps
against the reference's own Step(dt) (tests/golden/dyn_nh.npz)."""
import os

import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def test_dynamic_residual_tangent_and_diagonal_vs_oracle():
    from solidfem_gb300 import FemPhysicsMatrixFree
    from solidfem_gb300.mesh import box_lattice

    m = box_lattice(6, 2, 2, extent=(1.5, 0.5, 0.5), jitter=0.15, seed=3)
    fixed = m.face_nodes(0, 0)
    kw = dict(young=1e5, poisson=0.45, density=1070.0, gravity=(0, 0, -9.81), material=3)
    p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, **kw)
    o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, (0, 0, -9.81), 3)
    rng = np.random.default_rng(0)
    xs = m.nodes + rng.normal(size=m.nodes.shape) * 1e-3
    x = m.nodes + rng.normal(size=m.nodes.shape) * 1e-3
    xs[fixed] = m.nodes[fixed]
    x[fixed] = m.nodes[fixed]
    v = rng.normal(size=m.nodes.shape) * 0.1
    v[fixed] = 0.0
    p.set_positions(xs)
    p.begin_step()
    p.set_positions(x)
    p.set_velocities(v)
    p.set_time_step(0.01)
    np.testing.assert_allclose(p.get_velocities(), v, rtol=0, atol=0)
    mp = o.reshuffle_map()
    sh = lambda a: (lambda b: (b.__setitem__(mp, a), b)[1])(np.zeros_like(a))  # noqa: E731
    o.set_positions_shuffled(sh(x))
    o.set_start_shuffled(sh(xs))
    o.set_velocities_shuffled(sh(v))
    o.set_time_step(0.01)
    r_g, r_o = p.ComputeGradients().ravel(), o.gradients()
    assert rel(r_g, r_o) <= 1e-12, rel(r_g, r_o)
    d = rng.normal(size=3 * o.n_free)
    assert rel(p.MatrixVectorMultiply(d).ravel(), o.matvec(d)) <= 1e-12
    assert rel(p.jacobi_diagonal().ravel(), o.jacobi_diagonal()) <= 1e-12
    p.set_time_step(0.0)  # back to the static problem
    o.set_time_step(0.0)
    assert rel(p.ComputeGradients().ravel(), o.gradients()) <= 1e-12


def _golden():
    return np.load(os.path.join(HERE, "golden", "dyn_nh.npz"))


def _body(g, precision="fp64"):
    from solidfem_gb300 import FemPhysicsMatrixFree

    return FemPhysicsMatrixFree(g["tets"], g["nodes"], g["fixed"], young=float(g["young"]), poisson=float(g["poisson"]),
                                density=float(g["density"]), gravity=g["gravity"], material=int(g["material"]),
                                precision=precision)


def test_explicit_steps_match_reference():
    g = _golden()
    p = _body(g)
    for k in range(int(g["steps"])):
        p.Step(float(g["dt"]), simtype=2, substeps=int(g["explicit_substeps"]))
        x, v = p.get_positions(), p.get_velocities()
        ex = np.abs(x - g["explicit_positions"][k]).max()
        ev = np.abs(v - g["explicit_velocities"][k]).max() / np.abs(g["explicit_velocities"][k]).max()
        assert ex <= 1e-12 and ev <= 1e-10, (k, ex, ev)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_implicit_steps_match_reference(precision):
    g = _golden()
    p = _body(g, precision)
    u_prev = np.zeros_like(g["nodes"])
    for k in range(int(g["steps"])):
        st = p.Step(float(g["dt"]), simtype=3, substeps=1, rel_tol=1e-12 if precision == "fp64" else 1e-10)
        assert st["status"] == 0, (k, st)
        x, v = p.get_positions(), p.get_velocities()
        u_ref = g["implicit_positions"][k] - g["nodes"]
        err = np.linalg.norm(x - g["implicit_positions"][k]) / np.linalg.norm(u_ref - u_prev)
        errv = rel(v, g["implicit_velocities"][k])
        print(f"{precision} step {k}: displacement-increment error {err:.2e}, velocity error {errv:.2e}, {st}")
        assert err <= (1e-8 if precision == "fp64" else 1e-6) and errv <= (1e-8 if precision == "fp64" else 1e-6)
        u_prev = u_ref


def test_nonlinearfem_implicit_and_explicit():
    from solidfem_gb300.pysolidfem import NonlinearFEM

    g = _golden()
    for simtype, sub in ((3, 1), (2, 10)):
        sim = NonlinearFEM(g["tets"], g["nodes"], g["fixed"],
                           {"young": 1e5, "poisson": 0.45, "density": 1070.0, "simtype": simtype, "substeps": sub,
                            "gravity": -9.81, "zup": True, "tol": 1e-9, "maxiter": 50})
        sim.step(float(g["dt"]))
        key = "implicit_positions" if simtype == 3 else "explicit_positions"
        ref = g[key][0]
        assert np.abs(sim.get_nodes() - ref).max() <= 1e-6 * np.abs(ref - g["nodes"]).max(), simtype
