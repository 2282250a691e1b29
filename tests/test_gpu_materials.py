"""The other MaterialModelType values (neo-Hookean (Ogden), distortional linear / Mooney / NH2 /
NH3 / Bonet-Wood / Ogden / NH6 / NH7) on the GPU in FP64, against the reference's own outputs
(tests/golden/variant_<m>.npz): stress, gradients, energy, tangent diagonal and assembled
tangent; the matrix-free product against the reference's assembled tangent times a vector."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def rel(a, b):
    b = np.ravel(b)
    return np.abs(np.ravel(a) - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("mat", list(range(4, 13)))
def test_variant_material_matches_reference(mat):
    from solidfem_gb300 import FemPhysicsMatrixFree

    g = np.load(os.path.join(HERE, "golden", f"variant_{mat}.npz"))
    p = FemPhysicsMatrixFree(g["tets"], g["nodes"], g["fixed"], young=float(g["young"]), poisson=float(g["poisson"]),
                             density=float(g["density"]), gravity=g["gravity"], material=mat)
    p.set_positions(g["pos_shuffled"][g["map"]])
    assert rel(p.element_stress(), g["stress"]) <= 1e-12
    assert rel(p.ComputeGradients(), g["grad"]) <= 1e-12
    e_el = p.ComputeElasticEnergy()
    assert abs(e_el - float(g["energy"])) <= 1e-12 * max(abs(float(g["energy"])), 1.0)
    assert rel(p.jacobi_diagonal(), g["diag"]) <= 1e-12
    assert rel(p.get_hessian(), g["K"]) <= 1e-12
    d = np.random.default_rng(mat).normal(size=g["K"].shape[0])
    assert rel(p.MatrixVectorMultiply(d), g["K"] @ d) <= 1e-12


def test_variant_materials_need_fp64():
    from solidfem_gb300 import FemPhysicsMatrixFree, SfemError
    from solidfem_gb300.mesh import box_lattice

    m = box_lattice(2, 1, 1)
    with pytest.raises(SfemError):
        FemPhysicsMatrixFree(m.tets, m.nodes, m.face_nodes(0, 0), material=7, precision="fp32")
