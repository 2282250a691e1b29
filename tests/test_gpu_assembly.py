"""Assembled tangent on the GPU (block CSR, 3 x 3 blocks) against the reference's own
ElasticEnergy::AssembleStiffnessMatrix (tests/golden/tangent_<mat>.npz) and against the
matrix-free product."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("name", ["linear", "stvk", "corot", "nh"])
def test_assembled_tangent_matches_reference(name):
    from solidfem_gb300 import FemPhysicsMatrixFree

    g = np.load(os.path.join(HERE, "golden", f"tangent_{name}.npz"))
    p = FemPhysicsMatrixFree(g["tets"], g["nodes"], g["fixed"], young=float(g["young"]), poisson=float(g["poisson"]),
                             density=float(g["density"]), gravity=(0, 0, -9.81), material=int(g["material"]))
    x = g["pos_shuffled"][g["map"]]  # original node order
    p.set_positions(x)
    K = p.get_hessian()
    err = np.abs(K - g["K"]).max() / np.abs(g["K"]).max()
    print(f"{name}: assembled tangent vs reference {err:.2e}, {p.get_hessian_sparse().nnz // 9} blocks")
    assert err <= 1e-12
    d = np.random.default_rng(1).normal(size=K.shape[0])
    mf = p.MatrixVectorMultiply(d).ravel()
    assert np.linalg.norm(p.tangent_matvec(d) - mf) <= 1e-12 * np.linalg.norm(mf)


def test_assembled_tangent_includes_mass_term_for_dynamics():
    from solidfem_gb300 import FemPhysicsMatrixFree

    g = np.load(os.path.join(HERE, "golden", "tangent_nh.npz"))
    p = FemPhysicsMatrixFree(g["tets"], g["nodes"], g["fixed"], young=1e5, poisson=0.45, density=1070.0,
                             gravity=(0, 0, -9.81), material=3)
    K0 = p.get_hessian()
    p.set_time_step(0.01)
    K1 = p.get_hessian()
    dm = np.diag(K1 - K0)
    assert np.abs((K1 - K0) - np.diag(dm)).max() == 0.0
    ones = np.ones(K0.shape[0])
    total_mass = float(p.MatrixVectorMultiply(ones).sum() - (K0 @ ones).sum()) / 3 * 0.01 ** 2
    np.testing.assert_allclose(dm.sum() / 3 * 0.01 ** 2, total_mass, rtol=1e-10)
