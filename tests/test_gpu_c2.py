"""The large plain-vs-mixed-precision workload at full size: box [0,8]x[0,2]x[0,2], 128x32x32 hexes x 6 tets
(140,481 nodes / 786,432 tets), corotational and neo-Hookean, E = 1e6 Pa, nu = 0.4, 500 Pa
traction in -z on the x = 8 face, x = 0 clamped.  FP64 element kernels + CG against FP32
element kernels + CG with the FP64 Newton residual; the FP64 equilibrium is certified by the
oracle's own FP64 residual (a size-independent property: no CPU solve at this size)."""
import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("material", [2, 3])
def test_c2_fp32_vs_fp64_and_oracle_residual(material):
    from solidfem_gb300 import FemPhysicsMatrixFree
    from solidfem_gb300.mesh import box_lattice, lumped_face_load

    m = box_lattice(128, 32, 32, extent=(8.0, 2.0, 2.0))
    assert m.n_nodes == 140481 and m.n_tets == 786432
    fixed = m.face_nodes(0, 0)
    f = lumped_face_load(m, 0, 1, (0.0, 0.0, -500.0))
    kw = dict(young=1e6, poisson=0.4, density=1070.0, gravity=(0, 0, 0), material=material, tangent="exact")
    res = {}
    for prec in ("fp64", "fp32"):
        p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, precision=prec, **kw)
        p.set_nodal_loads(f)
        st = p.newton_solve(rel_tol=1e-10, max_newton=60)
        assert st["status"] == 0, (prec, st)
        res[prec] = (p.get_positions() - m.nodes, st)
    u64, st64 = res["fp64"]
    u32, st32 = res["fp32"]
    err = np.linalg.norm(u32 - u64) / np.linalg.norm(u64)
    print(f"C2 material {material}: FP64 {st64['seconds']:.2f} s ({st64['newton_iters']} Newton, "
          f"{st64['cg_iters']} CG); FP32-refined {st32['seconds']:.2f} s ({st32['newton_iters']} Newton, "
          f"{st32['cg_iters']} CG); displacement error FP32 vs FP64 {err:.2e}")
    assert err <= 1e-6
    o = Oracle(m.nodes, m.tets, fixed, 1e6, 0.4, 1070.0, (0, 0, 0), material)
    o.set_nodal_loads(f)
    r0 = np.linalg.norm(o.gradients())
    o.set_positions_shuffled(np.zeros(1) if False else _shuffled(o, m.nodes + u64))
    r = np.linalg.norm(o.gradients())
    print(f"oracle FP64 residual at the GPU FP64 equilibrium: {r / r0:.2e} of |r0|")
    assert r <= 1e-9 * r0


def _shuffled(o, x):
    out = np.zeros_like(x)
    out[o.reshuffle_map()] = x
    return out
