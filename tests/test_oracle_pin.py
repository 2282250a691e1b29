"""Pin the oracle against the reference's own sources compiled unmodified
(oracle/_ref).  Runs only where the reference tree is present."""
import numpy as np
import pytest

import os

from oracle.oracle import Oracle, RefHarness
from solidfem_gb300.mesh import box_lattice, lumped_face_load

HERE = os.path.dirname(os.path.abspath(__file__))

pytestmark = pytest.mark.skipif(not RefHarness.available(), reason="reference tree not present")


@pytest.mark.parametrize("material", [0, 1, 2, 3])
@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_bit_identical_to_reference(material, seed):
    rng = np.random.default_rng(seed)
    m = box_lattice(5, 3, 2, extent=(2.0, 1.0, 0.7), jitter=0.25, seed=seed)
    fixed = m.face_nodes(0, 0)
    # flip some tets to exercise the orientation fix of FemBody::Prepare
    tets = m.tets.copy()
    flip = rng.random(len(tets)) < 0.3
    tets[flip, 0], tets[flip, 1] = m.tets[flip, 1], m.tets[flip, 0]
    ref = RefHarness(m.nodes, tets, fixed, 2e5, 0.42, 1000.0, -9.81, True, material)
    orc = Oracle(m.nodes, tets, fixed, 2e5, 0.42, 1000.0, (0, 0, -9.81), material)
    ref.set_force_fraction(1.0)
    f = lumped_face_load(m, 0, 1, (10.0, 20.0, -500.0))
    ref.set_nodal_loads(f)
    orc.set_nodal_loads(f)
    assert np.array_equal(ref.reshuffle_map(), orc.reshuffle_map())
    assert np.array_equal(ref.tets(), orc.tets())
    x = orc.positions_shuffled() + 0.03 * rng.normal(size=(m.n_nodes, 3))
    x[: orc.n_bcs] = orc.positions_shuffled()[: orc.n_bcs]
    ref.set_positions_shuffled(x)
    orc.set_positions_shuffled(x)
    d = rng.normal(size=3 * orc.n_free)
    np.testing.assert_array_equal(ref.gradients(), orc.gradients())
    np.testing.assert_array_equal(ref.matvec(d), orc.matvec(d))
    np.testing.assert_array_equal(ref.jacobi_diagonal(), orc.jacobi_diagonal())
    np.testing.assert_array_equal(ref.element_stress(), orc.element_stress())
    assert ref.elastic_energy() == orc.elastic_energy()
    for a, b in zip(ref.force_param_grads(), orc.force_param_grads()):
        np.testing.assert_array_equal(a, b)


def test_follower_pressure_bit_identical_to_reference():
    rng = np.random.default_rng(5)
    m = box_lattice(5, 3, 2, extent=(2.0, 1.0, 0.7), jitter=0.25, seed=4)
    fixed = m.face_nodes(0, 0)
    tris = np.concatenate([m.face_triangles(2, 1), m.face_triangles(0, 1)])
    ref = RefHarness(m.nodes, m.tets, fixed, 2e5, 0.42, 1000.0, -9.81, True, 3)
    orc = Oracle(m.nodes, m.tets, fixed, 2e5, 0.42, 1000.0, (0, 0, -9.81), 3)
    ref.set_force_fraction(1.0)
    ref.set_pressure_surface(tris, 1500.0)
    orc.set_pressure_surface(tris, 1500.0)
    x = orc.positions_shuffled() + 0.02 * rng.normal(size=(m.n_nodes, 3))
    x[: orc.n_bcs] = orc.positions_shuffled()[: orc.n_bcs]
    ref.set_positions_shuffled(x)
    orc.set_positions_shuffled(x)
    np.testing.assert_array_equal(ref.gradients(), orc.gradients())


# ---- dynamics: FemPhysicsMatrixFree::ComputeGradients / MatrixVectorMultiply with mTimeStep != 0
# (Source/FemPhysicsMatrixFree.cpp:523-560) and SubStep (:371-387) ----
@pytest.mark.skipif(not RefHarness.available(), reason="reference not built here")
def test_dynamic_terms_bit_identical_to_reference():
    m = box_lattice(6, 2, 2, extent=(1.5, 0.5, 0.5), jitter=0.15, seed=3)
    fixed = m.face_nodes(0, 0)
    ref = RefHarness(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, -9.81, True, 3)
    orc = Oracle(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, (0, 0, -9.81), 3)
    ref.set_force_fraction(1.0)
    rng = np.random.default_rng(0)
    x0 = ref.positions_shuffled().copy()
    x = x0 + rng.normal(size=x0.shape) * 1e-3
    x[:ref.n_bcs] = x0[:ref.n_bcs]
    xs = x0 + rng.normal(size=x0.shape) * 1e-3
    v = rng.normal(size=x0.shape) * 0.1
    ref.set_positions_shuffled(x.ravel())
    orc.set_positions_shuffled(x)
    for o in (ref, orc):
        o.set_time_step(0.01)
        o.set_velocities_shuffled(v)
        o.set_start_shuffled(xs)
    np.testing.assert_array_equal(orc.gradients(), ref.gradients())
    d = rng.normal(size=3 * ref.n_free)
    np.testing.assert_array_equal(orc.matvec(d), ref.matvec(d))
    # explicit substeps: the reference's Step(dt) with ST_EXPLICIT and 5 substeps
    ref2 = RefHarness(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, -9.81, True, 3)
    orc2 = Oracle(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, (0, 0, -9.81), 3)
    ref2.set_sim(2, 5)
    ref2.step_dt(0.005)
    for _ in range(5):
        orc2.explicit_substep(0.001)
    np.testing.assert_array_equal(orc2.positions_shuffled(), ref2.positions_shuffled())
    np.testing.assert_array_equal(orc2.velocities_shuffled(), ref2.velocities_shuffled())


def test_dynamics_golden_is_consistent_with_the_oracle():
    """The reference's implicit steps in tests/golden/dyn_nh.npz solve the backward-Euler
    residual of the oracle; its explicit steps equal the oracle's substeps."""
    g = np.load(os.path.join(HERE, "golden", "dyn_nh.npz"))
    o = Oracle(g["nodes"], g["tets"], g["fixed"], 1e5, 0.45, 1070.0, g["gravity"], 3)
    mp = o.reshuffle_map()
    dt = float(g["dt"])
    xprev = g["nodes"]
    vprev = np.zeros_like(xprev)
    for k in range(int(g["steps"])):
        x, v = g["implicit_positions"][k], g["implicit_velocities"][k]
        xs = np.zeros_like(x)
        xs[mp] = xprev
        vs = np.zeros_like(x)
        vs[mp] = vprev
        xx = np.zeros_like(x)
        xx[mp] = x
        o.set_positions_shuffled(xx)
        o.set_start_shuffled(xs)
        o.set_velocities_shuffled(vs)
        o.set_time_step(dt)
        r = o.gradients()
        o.set_positions_shuffled(xs)
        r0 = o.gradients()
        assert np.linalg.norm(r) <= 1e-8 * np.linalg.norm(r0), (k, np.linalg.norm(r), np.linalg.norm(r0))
        np.testing.assert_allclose(v, (x - xprev) / dt, rtol=0, atol=1e-12 * max(1.0, np.abs(v).max()))
        xprev, vprev = x, v
    o2 = Oracle(g["nodes"], g["tets"], g["fixed"], 1e5, 0.45, 1070.0, g["gravity"], 3)
    for k in range(int(g["steps"])):
        for _ in range(int(g["explicit_substeps"])):
            o2.explicit_substep(dt / int(g["explicit_substeps"]))
        np.testing.assert_allclose(o2.positions(), g["explicit_positions"][k], rtol=0, atol=1e-14)


# ---- the other MaterialModelType values (ElasticEnergy.cpp:40-112, 188-254, 412-479) ----
@pytest.mark.skipif(not RefHarness.available(), reason="reference not built here")
@pytest.mark.parametrize("mat", list(range(4, 13)))
def test_variant_materials_bit_identical_to_reference(mat):
    m = box_lattice(4, 2, 2, extent=(1.0, 0.5, 0.5), jitter=0.15, seed=5)
    fixed = m.face_nodes(0, 0)
    ref = RefHarness(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, -9.81, True, mat)
    orc = Oracle(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, (0, 0, -9.81), mat)
    ref.set_force_fraction(1.0)
    rng = np.random.default_rng(mat)
    x = ref.positions_shuffled() + rng.normal(size=(m.n_nodes, 3)) * 0.01
    x[:ref.n_bcs] = ref.positions_shuffled()[:ref.n_bcs]
    ref.set_positions_shuffled(x.ravel())
    orc.set_positions_shuffled(x)
    np.testing.assert_array_equal(orc.element_stress().ravel(), ref.element_stress().ravel())
    np.testing.assert_array_equal(orc.gradients(), ref.gradients())
    assert orc.elastic_energy() == ref.elastic_energy()
    np.testing.assert_array_equal(orc.jacobi_diagonal(), ref.jacobi_diagonal())
    for a, b in zip(orc.force_param_grads(), ref.force_param_grads()):
        np.testing.assert_array_equal(a, b)
