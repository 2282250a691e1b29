"""GPU parity: the CUDA library (through the C ABI) against the golden fixtures
produced by the reference's own code and against the oracle on seeded inputs.

Tolerances (FP64 mode): element-level results (forces, Hessian-vector product,
Jacobi diagonal, stress, energy, parameter gradients) <= 1e-12 relative in the
2-norm -- the GPU sums in the same element order but contracts multiply-adds
and uses its own log/sqrt, so results differ from the reference by rounding
only.  Equilibria: relative displacement error <= 1e-6 against the reference.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from tests.conftest import load_golden

pytestmark = pytest.mark.gpu

ELEM_TOL = 1e-12
CASES = ["box2_nh.npz", "lattice_linear.npz", "lattice_stvk.npz", "lattice_corot.npz", "lattice_nh.npz"]


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


def gpu_problem(g, precision="fp64", **kw):
    from solidfem_gb300 import FemPhysicsMatrixFree

    p = FemPhysicsMatrixFree(g["tets"], g["nodes"], g["fixed"], young=float(g["young"]),
                             poisson=float(g["poisson"]), density=float(g["density"]), gravity=g["gravity"],
                             material=int(g["material"]), precision=precision, **kw)
    if "loads" in g:
        p.set_nodal_loads(g["loads"])
    return p


@pytest.mark.parametrize("case", CASES)
def test_element_level_vs_reference_fixture(case):
    g = load_golden(case)
    p = gpu_problem(g)
    assert np.array_equal(p.reshuffle_map(), g["map"])
    nbc = p.n_bcs
    assert rel(p.ComputeGradients(), g["grad_rest"]) <= ELEM_TOL
    p.set_free_positions(g["pos_shuffled"][nbc:])
    checks = {
        "grad": p.ComputeGradients(),
        "matvec": p.MatrixVectorMultiply(g["d"]),
        "diag": p.jacobi_diagonal(),
        "stress": p.element_stress(),
        "energy": np.array(p.ComputeElasticEnergy()),
    }
    for name, val in checks.items():
        assert rel(val, g[name]) <= ELEM_TOL, (case, name, rel(val, g[name]))
    gmu, gl, grho = p.GetForceParamGrads()
    for val, ref in [(gmu, g["gmu"]), (gl, g["glambda"]), (grho, g["grho"])]:
        if np.linalg.norm(ref) == 0:
            assert np.linalg.norm(val) == 0
        else:
            assert rel(val, ref) <= ELEM_TOL
    # the same positions read back in original node order
    pos = p.get_positions()
    m = g["map"]
    np.testing.assert_array_equal(pos, g["pos_shuffled"][m])


@pytest.mark.parametrize("material", [0, 1, 2, 3])
def test_matvec_and_gradients_vs_oracle_random(material):
    from solidfem_gb300.mesh import box_lattice, lumped_face_load

    rng = np.random.default_rng(100 + material)
    m = box_lattice(12, 5, 4, extent=(3.0, 1.0, 0.8), jitter=0.2, seed=material)
    fixed = m.face_nodes(0, 0)
    f = lumped_face_load(m, 2, 1, (0.0, 0.0, -700.0))
    orc = Oracle(m.nodes, m.tets, fixed, 3e5, 0.43, 1100.0, (0.0, -2.0, -9.81), material)
    orc.set_nodal_loads(f)
    g = dict(tets=m.tets, nodes=m.nodes, fixed=fixed, young=3e5, poisson=0.43, density=1100.0,
             gravity=np.array([0.0, -2.0, -9.81]), material=material, loads=f)
    p = gpu_problem(g)
    x = orc.free_positions() + 0.02 * rng.normal(size=3 * orc.n_free)
    orc.set_free_positions(x)
    p.set_free_positions(x)
    for _ in range(3):
        d = rng.normal(size=3 * orc.n_free)
        assert rel(p.MatrixVectorMultiply(d), orc.matvec(d)) <= ELEM_TOL
    assert rel(p.ComputeGradients(), orc.gradients()) <= ELEM_TOL
    assert rel(p.jacobi_diagonal(), orc.jacobi_diagonal()) <= ELEM_TOL
    assert abs(p.ComputeEnergy() - orc.total_energy()) <= ELEM_TOL * abs(orc.elastic_energy())
    assert p.count_inverted() == orc.count_inverted() == 0
    # per-element Young's modulus (extension): the oracle scales mu and lambda per element
    ye = 3e5 * np.exp(0.5 * rng.normal(size=m.n_tets))
    p.set_element_youngs(ye)
    orc.set_element_scale(ye / 3e5)
    d = rng.normal(size=3 * orc.n_free)
    assert rel(p.MatrixVectorMultiply(d), orc.matvec(d)) <= ELEM_TOL
    assert rel(p.ComputeGradients(), orc.gradients()) <= ELEM_TOL


def test_fp32_matvec_error_is_reported():
    """FP32 element kernels: error against the FP64 oracle is stated, not gated tightly."""
    from solidfem_gb300.mesh import box_lattice

    rng = np.random.default_rng(5)
    m = box_lattice(12, 4, 4, extent=(3.0, 1.0, 1.0), jitter=0.2, seed=5)
    fixed = m.face_nodes(0, 0)
    orc = Oracle(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, (0, 0, -9.81), 3)
    g = dict(tets=m.tets, nodes=m.nodes, fixed=fixed, young=1e5, poisson=0.45, density=1070.0,
             gravity=np.array([0, 0, -9.81]), material=3)
    p = gpu_problem(g, precision="fp32")
    # a state near rest, where the neo-Hookean tangent is positive definite
    x = orc.free_positions() + 1e-4 * rng.normal(size=3 * orc.n_free)
    orc.set_free_positions(x)
    p.set_free_positions(x)
    b = rng.normal(size=3 * orc.n_free)
    # FP32 PCG solve vs FP64 oracle PCG solve of the same system
    xg, st = p.pcg(b, rel_tol=1e-5, max_iters=5000)
    xo, its, _ = orc.pcg(b, diag=orc.jacobi_diagonal(), tol=1e-10, max_iters=20000)
    err = rel(xg, xo)
    print(f"fp32 PCG: iters={st['iters']} rel err vs fp64 oracle = {err:.2e}")
    assert err < 1e-3


def _u_rel(pos, g):
    u = pos - g["nodes"]
    uref = g["eq_positions"] - g["nodes"]
    return np.linalg.norm(u - uref) / np.linalg.norm(uref)


def test_c1_equilibrium_matches_reference_newton_ls():
    """16x4x4 cantilever under gravity (large deformation): the GPU Newton-PCG (FP64)
    reaches the reference SolveNewtonLS equilibrium."""
    g = load_golden("c1_newton_ls.npz")
    p = gpu_problem(g)
    st = p.newton_solve(rel_tol=1e-10, max_newton=200, load_steps=1)
    assert st["status"] == 0, st
    err = _u_rel(p.get_positions(), g)
    print("C1", st, "disp rel err", err)
    assert err <= 1e-6


@pytest.mark.parametrize("case", ["box2_nh.npz", "c2s_nh.npz"])
def test_equilibrium_matches_reference(case):
    g = load_golden(case)
    p = gpu_problem(g)
    st = p.newton_solve(rel_tol=1e-11, max_newton=100)
    assert st["status"] == 0, st
    assert _u_rel(p.get_positions(), g) <= 1e-6


def test_fp32_mixed_precision_reaches_fp64_residual():
    g = load_golden("c2s_nh.npz")
    p = gpu_problem(g, precision="fp32")
    st = p.newton_solve(rel_tol=1e-10, max_newton=100)
    assert st["status"] == 0, st
    err = _u_rel(p.get_positions(), g)
    print("fp32 mixed: disp rel err vs reference", err, st)
    assert err <= 1e-6


def test_corotational_equilibrium_with_exact_tangent():
    """Corotational: the reference's force fixes the equilibrium; the exact derivative of that
    force (SFEM_TANGENT_EXACT) gives Newton its quadratic convergence back."""
    g = load_golden("c2s_corot.npz")
    p = gpu_problem(g, tangent="exact")
    st = p.newton_solve(rel_tol=1e-11, max_newton=60)
    assert st["status"] == 0, st
    assert _u_rel(p.get_positions(), g) <= 1e-6


@pytest.mark.parametrize("material", [0, 1, 2, 3])
def test_exact_tangent_matches_finite_differences_of_gpu_residual(material):
    from solidfem_gb300.mesh import box_lattice

    rng = np.random.default_rng(7)
    m = box_lattice(6, 3, 3, extent=(2.0, 1.0, 1.0), jitter=0.2, seed=2)
    g = dict(tets=m.tets, nodes=m.nodes, fixed=m.face_nodes(0, 0), young=1e5, poisson=0.4, density=1000.0,
             gravity=np.zeros(3), material=material)
    p = gpu_problem(g, tangent="exact")
    x = p.get_free_positions().ravel() + 0.05 * rng.normal(size=3 * p.n_free)
    d = rng.normal(size=3 * p.n_free)
    h = 1e-6
    p.set_free_positions(x + h * d)
    rp = p.ComputeGradients().ravel()
    p.set_free_positions(x - h * d)
    rm = p.ComputeGradients().ravel()
    p.set_free_positions(x)
    fd = -(rp - rm) / (2 * h)
    assert rel(p.MatrixVectorMultiply(d), fd) <= 1e-7


def test_follower_pressure_gradients_vs_oracle():
    from solidfem_gb300.mesh import box_lattice

    rng = np.random.default_rng(9)
    m = box_lattice(10, 4, 3, extent=(2.5, 1.0, 0.75), jitter=0.2, seed=6)
    fixed = m.face_nodes(0, 0)
    tris = np.concatenate([m.face_triangles(2, 1), m.face_triangles(0, 1)])
    orc = Oracle(m.nodes, m.tets, fixed, 2e5, 0.42, 1000.0, (0, 0, -9.81), 3)
    orc.set_pressure_surface(tris, 1500.0)
    g = dict(tets=m.tets, nodes=m.nodes, fixed=fixed, young=2e5, poisson=0.42, density=1000.0,
             gravity=np.array([0, 0, -9.81]), material=3)
    p = gpu_problem(g)
    p.SetBoundaryConditionsSurface(tris, 1500.0)
    x = orc.free_positions() + 0.02 * rng.normal(size=3 * orc.n_free)
    orc.set_free_positions(x)
    p.set_free_positions(x)
    assert rel(p.ComputeGradients(), orc.gradients()) <= ELEM_TOL
    # a static solve with the follower load converges (residual line search; the pressure
    # stiffness is not in the product, as in the reference, so Newton converges linearly)
    from solidfem_gb300 import FemPhysicsMatrixFree

    q = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, young=2e7, poisson=0.42, density=1000.0,
                             gravity=(0, 0, -9.81), material=3)
    q.SetBoundaryConditionsSurface(tris, 1500.0)
    st = q.newton_solve(rel_tol=1e-9, max_newton=100)
    assert st["status"] == 0, st


def test_node_arrays_round_trip_in_caller_order():
    """Positions, velocities and loads cross the C ABI in the caller's node order and are permuted
    to the reshuffled order on the device: set/get round trips, the fixed block of velocities,
    and a load placed on one node showing up in that node's residual."""
    g = load_golden("lattice_nh.npz")
    p = gpu_problem(g)
    n = p.n_nodes
    rng = np.random.default_rng(3)
    x = np.asarray(g["nodes"], dtype=np.float64) + 1e-3 * rng.normal(size=(n, 3))
    p.set_positions(x)
    assert np.allclose(p.get_positions(), x, rtol=0, atol=4 * np.finfo(np.float64).eps * np.abs(x).max())
    out = np.empty((n, 3))
    assert p.get_positions(out=out) is out and np.array_equal(out, p.get_positions())
    v = rng.normal(size=(n, 3))
    p.set_velocities(v)
    vg = p.get_velocities()
    fixed = np.asarray(g["fixed"])
    free = np.setdiff1d(np.arange(n), fixed)
    assert np.array_equal(vg[free], v[free]) and not vg[fixed].any()
    # a unit load on one free node moves exactly that node's entry of the residual
    p.set_positions(np.asarray(g["nodes"], dtype=np.float64))
    p.set_nodal_loads(np.zeros((n, 3)))
    r0 = p.ComputeGradients()
    f = np.zeros((n, 3))
    node = int(free[len(free) // 2])
    f[node] = (1.0, -2.0, 0.5)
    p.set_nodal_loads(f)
    d = p.ComputeGradients() - r0
    row = int(p.reshuffle_map()[node]) - p.n_bcs
    assert np.allclose(d[row], f[node]) and np.abs(np.delete(d, row, axis=0)).max() == 0.0
