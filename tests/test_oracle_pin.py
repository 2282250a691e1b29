"""Pin the oracle against the reference's own sources compiled unmodified
(oracle/_ref).  Runs only where the reference tree is present."""
import numpy as np
import pytest

from oracle.oracle import Oracle, RefHarness
from solidfem_gb300.mesh import box_lattice, lumped_face_load

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
