"""The assembled FP32 operator of the Krylov solves (sliced-ELL tangent, `sfem_set_operator`)
against the matrix-free patch product: the same linear solves, the same equilibria, with Jacobi
and with the learned preconditioner, statically and in implicit dynamics."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def slab(nx=24, ny=8, nz=8, material=3, **kw):
    from solidfem_gb300 import FemPhysicsMatrixFree
    from solidfem_gb300.mesh import box_lattice, random_top_traction

    m = box_lattice(nx, ny, nz, extent=(4.0 * nx / 256, 1.0 * ny / 64, 1.0 * nz / 64), jitter=0.2, seed=0)
    fixed = m.face_nodes(2, 0)
    p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, young=1e5, poisson=0.49, density=1070.0,
                             gravity=(0, 0, 0), material=material, precision="fp32", **kw)
    p.set_nodal_loads(random_top_traction(m, seed=7))
    return m, p


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


@pytest.mark.parametrize("material", [0, 1, 2, 3])
def test_pcg_solution_matches_matrix_free(material):
    """K x = b at a deformed state: FP32 Jacobi-PCG to 1e-6 with either operator."""
    m, p = slab(material=material)
    rng = np.random.default_rng(material)
    # a small random state (strains ~ 1e-3: the StVK and corotational tangents stay definite)
    p.set_positions(m.nodes + 2e-5 * rng.normal(size=m.nodes.shape))
    b = rng.normal(size=(p.n_free, 3))
    x_mf, st_mf = p.pcg(b, rel_tol=1e-6, max_iters=20000)
    p.set_operator("assembled")
    x_as, st_as = p.pcg(b, rel_tol=1e-6, max_iters=20000)
    p.set_operator("matrix-free")
    # both solutions against the handle's own product (FP32 solves to 1e-6: the two solutions may
    # differ by the residual tolerance times the condition number)
    res = [rel(p.MatrixVectorMultiply(x).ravel(), b.ravel()) for x in (x_mf, x_as)]
    print(f"material {material}: iterations {st_mf['iters']} / {st_as['iters']}, solution rel diff "
          f"{rel(x_as, x_mf):.2e}, residuals {res[0]:.2e} / {res[1]:.2e}")
    assert st_mf["status"] == 0 and st_as["status"] == 0
    # FP32 solves stop near the FP32 floor of the true residual: the two operators reach the same one
    assert rel(x_as, x_mf) < 1e-3 and max(res) < 1e-3 and res[1] <= 1.5 * res[0] + 1e-6
    assert abs(st_as["iters"] - st_mf["iters"]) <= max(5, st_mf["iters"] // 20)


@pytest.mark.parametrize("precond", ["jacobi", "learned"])
def test_newton_equilibrium_matches_matrix_free(precond):
    import os

    from solidfem_gb300 import PC_JACOBI, PC_LEARNED
    from solidfem_gb300.learned import LearnedPreconditioner

    m, p = slab(32, 8, 8)
    pc = PC_JACOBI
    if precond == "learned":
        net = LearnedPreconditioner(p)
        net.load(os.path.join(os.path.dirname(__file__), "..", "solidfem_gb300", "data", "gnn_slab.bin"))
        pc = PC_LEARNED
    st_mf = p.newton_solve(rel_tol=1e-8, precond=pc)
    x_mf = p.get_positions()
    p.set_positions(m.nodes)
    p.set_operator("assembled")
    st_as = p.newton_solve(rel_tol=1e-8, precond=pc)
    x_as = p.get_positions()
    print(f"{precond}: matrix-free {st_mf}\n  assembled {st_as}")
    assert st_mf["status"] == 0 and st_as["status"] == 0 and st_as["rel_res"] <= 1e-8
    u_mf, u_as = x_mf - m.nodes, x_as - m.nodes
    assert rel(u_as, u_mf) < 1e-6
    assert st_as["cg_iters"] <= 1.1 * st_mf["cg_iters"] + 10


def test_implicit_step_matches_matrix_free():
    """Backward Euler: the mass term enters the assembled diagonal blocks."""
    from solidfem_gb300._native import SIM_IMPLICIT

    res = []
    for op in ("matrix-free", "assembled"):
        m, p = slab(16, 4, 4)
        p.set_operator(op)
        p.set_nodal_loads(None)
        p.set_velocities(np.tile([0.0, 0.0, -0.05], (m.nodes.shape[0], 1)))
        st = p.Step(dt=1e-3, simtype=SIM_IMPLICIT, substeps=2)
        res.append((p.get_positions() - m.nodes, st))
    (u_mf, st_mf), (u_as, st_as) = res
    print(st_mf, st_as, rel(u_as, u_mf))
    assert rel(u_as, u_mf) < 1e-6


@pytest.mark.parametrize("material", [1, 3])
def test_fp64_assembled_matches_matrix_free(material):
    """The FP64 assembled operator: a PCG solve to 1e-10 and the Newton equilibrium agree with the
    matrix-free FP64 product to rounding."""
    from solidfem_gb300 import FemPhysicsMatrixFree
    from solidfem_gb300.mesh import box_lattice, random_top_traction

    m = box_lattice(24, 8, 8, extent=(24 / 64, 8 / 64, 8 / 64), jitter=0.2, seed=0)
    fixed = m.face_nodes(2, 0)
    p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, young=1e5, poisson=0.45, density=1070.0,
                             gravity=(0, 0, 0), material=material, precision="fp64")
    p.set_nodal_loads(random_top_traction(m, seed=3))
    rng = np.random.default_rng(5)
    p.set_positions(m.nodes + 2e-5 * rng.normal(size=m.nodes.shape))
    b = rng.normal(size=(p.n_free, 3))
    x_mf, st_mf = p.pcg(b, rel_tol=1e-10, max_iters=50000)
    p.set_operator("assembled")
    x_as, st_as = p.pcg(b, rel_tol=1e-10, max_iters=50000)
    print(f"FP64 material {material}: PCG {st_mf['iters']} / {st_as['iters']}, rel diff {rel(x_as, x_mf):.2e}")
    assert st_mf["status"] == 0 and st_as["status"] == 0 and rel(x_as, x_mf) < 1e-7
    sols = []
    for op in ("matrix-free", "assembled"):
        p.set_operator(op)
        p.set_positions(m.nodes)
        st = p.newton_solve(rel_tol=1e-9)
        assert st["status"] == 0, (op, st)
        sols.append(p.get_positions() - m.nodes)
    print(f"  Newton displacement rel diff {rel(sols[1], sols[0]):.2e}")
    assert rel(sols[1], sols[0]) < 1e-8


def free_block_pattern(tets, rmap, nbc):
    """(row, column) free-node pairs of the assembled tangent: every pair of free nodes of a tet,
    in the handle's free-node numbering (rmap: caller index -> reshuffled index)."""
    t = rmap[tets].astype(np.int64) - nbc
    a = np.repeat(t, 4, axis=1).ravel()
    c = np.tile(t, (1, 4)).ravel()
    keep = (a >= 0) & (c >= 0)
    key = np.unique(a[keep] * (int(t.max()) + 1) + c[keep])
    return key // (int(t.max()) + 1), key % (int(t.max()) + 1)


def randomly_numbered_lattice():
    """The 64x24x24-hex lattice (40,625 nodes) and the same mesh under a random node numbering:
    (lattice mesh, fixed nodes, loads), (nodes, tets, fixed nodes, loads) renumbered, perm
    (node k of the renumbered mesh is node perm[k] of the lattice)."""
    from solidfem_gb300.mesh import box_lattice, random_top_traction

    m = box_lattice(64, 24, 24, extent=(1.0, 24 / 64, 24 / 64), jitter=0.2, seed=0)
    fixed = m.face_nodes(2, 0)
    loads = random_top_traction(m, seed=7)
    perm = np.random.default_rng(11).permutation(len(m.nodes))
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm))
    return (m, fixed, loads), (m.nodes[perm], inv[m.tets].astype(np.int32), inv[fixed], loads[perm]), perm


def test_randomly_numbered_mesh_32bit_indices():
    """A randomly numbered lattice of 40,625 nodes, where column differences and neighbour deltas no
    longer fit 16 bits: the sliced-ELL product keeps 32-bit columns (read back from the profile's
    bytes per block) and the learned preconditioner reads 32-bit neighbour indices.  Jacobi-PCG and
    the learned Newton solve agree with the matrix-free product, and the equilibrium with the one
    of the same mesh in lattice order."""
    import os

    from solidfem_gb300 import PC_LEARNED, FemPhysicsMatrixFree
    from solidfem_gb300.learned import LearnedPreconditioner

    (m, fixed, loads), (nodes_p, tets_p, fixed_p, loads_p), perm = randomly_numbered_lattice()
    weights = os.path.join(os.path.dirname(__file__), "..", "solidfem_gb300", "data", "gnn_slab.bin")

    def physics(nodes, tets, fx, f):
        p = FemPhysicsMatrixFree(tets, nodes, fx, young=1e5, poisson=0.49, density=1070.0, gravity=(0, 0, 0),
                                 material=3, precision="fp32")
        p.set_nodal_loads(f)
        return p

    p = physics(nodes_p, tets_p, fixed_p, loads_p)
    rows, cols = free_block_pattern(tets_p, p.reshuffle_map(), p.n_bcs)
    assert np.abs(cols - rows).max() > 32767

    # Jacobi-PCG at a deformed state, both operators
    rng = np.random.default_rng(3)
    p.set_positions(nodes_p + 2e-5 * rng.normal(size=nodes_p.shape))
    b = rng.normal(size=(p.n_free, 3))
    x_mf, st_mf = p.pcg(b, rel_tol=1e-6, max_iters=20000)
    p.set_operator("assembled")
    p.set_profiling(True)
    x_as, st_as = p.pcg(b, rel_tol=1e-6, max_iters=20000)
    prof = p.get_profile()
    p.set_profiling(False)
    p.set_operator("matrix-free")
    # the symmetric tangent streams its diagonal and upper blocks (36 B of values + c B of column each)
    # and per lower block a column (c B) and its mirror's block-slot (4 B)
    n_up, n_low = (len(rows) + p.n_free) // 2, (len(rows) - p.n_free) // 2
    col_bytes = (prof["algo_bytes_hvp"] - 48.0 * p.n_free - 36.0 * n_up - 4.0 * n_low) / (n_up + n_low)
    res = [rel(p.MatrixVectorMultiply(x).ravel(), b.ravel()) for x in (x_mf, x_as)]
    print(f"PCG iterations {st_mf['iters']} / {st_as['iters']}, column bytes {col_bytes:.3f}, "
          f"residuals {res[0]:.2e} / {res[1]:.2e}")
    assert abs(col_bytes - 4.0) < 1e-6
    assert st_mf["status"] == 0 and st_as["status"] == 0
    assert rel(x_as, x_mf) < 1e-3 and max(res) < 1e-3 and res[1] <= 1.5 * res[0] + 1e-6

    # the learned Newton solve: 32-bit neighbour indices, both operators, and lattice order
    net = LearnedPreconditioner(p)
    net.load(weights)
    assert net.graph_form()[0] == "index32"
    sols = []
    for op in ("matrix-free", "assembled"):
        p.set_operator(op)
        p.set_positions(nodes_p)
        st = p.newton_solve(rel_tol=1e-8, precond=PC_LEARNED)
        print(f"randomly numbered, {op}: {st}")
        assert st["status"] == 0 and st["rel_res"] <= 1e-8
        sols.append(p.get_positions() - nodes_p)
    q = physics(m.nodes, m.tets, fixed, loads)
    net_q = LearnedPreconditioner(q)
    net_q.load(weights)
    q.set_operator("assembled")
    st = q.newton_solve(rel_tol=1e-8, precond=PC_LEARNED)
    assert st["status"] == 0
    u_lattice = (q.get_positions() - m.nodes)[perm]
    print(f"displacement rel diffs: operators {rel(sols[1], sols[0]):.2e}, numberings {rel(sols[1], u_lattice):.2e}")
    assert rel(sols[1], sols[0]) < 1e-6 and rel(sols[1], u_lattice) < 1e-6


def test_randomly_numbered_mesh_fp64_assembled():
    """The FP64 assembled operator with 32-bit columns (the randomly numbered lattice): a Jacobi-PCG
    solve to 1e-10 agrees with the matrix-free FP64 product to rounding."""
    from solidfem_gb300 import FemPhysicsMatrixFree

    _, (nodes_p, tets_p, fixed_p, _), _ = randomly_numbered_lattice()
    p = FemPhysicsMatrixFree(tets_p, nodes_p, fixed_p, young=1e5, poisson=0.45, density=1070.0,
                             gravity=(0, 0, 0), material=3, precision="fp64")
    rows, cols = free_block_pattern(tets_p, p.reshuffle_map(), p.n_bcs)
    rng = np.random.default_rng(5)
    p.set_positions(nodes_p + 2e-5 * rng.normal(size=nodes_p.shape))
    b = rng.normal(size=(p.n_free, 3))
    x_mf, st_mf = p.pcg(b, rel_tol=1e-10, max_iters=50000)
    p.set_operator("assembled")
    p.set_profiling(True)
    x_as, st_as = p.pcg(b, rel_tol=1e-10, max_iters=50000)
    prof = p.get_profile()
    p.set_profiling(False)
    # stored blocks: 72 B of values + c B of column; lower blocks: c B of column + a 4 B mirror slot
    n_up, n_low = (len(rows) + p.n_free) // 2, (len(rows) - p.n_free) // 2
    col_bytes = (prof["algo_bytes_hvp"] - 96.0 * p.n_free - 72.0 * n_up - 4.0 * n_low) / (n_up + n_low)
    print(f"FP64 PCG {st_mf['iters']} / {st_as['iters']}, column bytes {col_bytes:.3f}, "
          f"rel diff {rel(x_as, x_mf):.2e}")
    assert abs(col_bytes - 4.0) < 1e-6
    assert st_mf["status"] == 0 and st_as["status"] == 0 and rel(x_as, x_mf) < 1e-7


def test_memory_limit_falls_back_without_leaking():
    """An assembly that cannot get its memory frees what it took, solves matrix-free, reports success
    with no error message, and does not retry every Newton step; lifting the cap assembles again."""
    from solidfem_gb300 import _native as nat

    m, p = slab(16, 8, 8)
    p.set_operator("assembled")
    st_ok = p.newton_solve(rel_tol=1e-8, max_newton=30)
    full, fb = p.operator_info()
    assert st_ok["status"] == 0 and full > 0 and not fb
    x_as = p.get_free_positions()
    p.set_operator("matrix-free")
    assert p.operator_info() == (0, False)
    p.set_positions(m.nodes)
    st_mf = p.newton_solve(rel_tol=1e-8, max_newton=30)
    x_mf = p.get_free_positions()
    # caps that fail at the first and at the last allocation of the assembly
    for cap in (1024, full - 1):
        p.set_operator("assembled")
        p.set_operator_memory_limit(cap)
        p.set_positions(m.nodes)
        st = p.newton_solve(rel_tol=1e-8, max_newton=30)
        assert st["status"] == 0 and st["newton_iters"] >= 2
        assert p.operator_info() == (0, True), p.operator_info()
        assert nat.load().sfem_last_error() in (b"", None)
        # the same iterates as the matrix-free solve: the fallback is that solve
        assert st["cg_iters"] == st_mf["cg_iters"]
        assert rel(p.get_free_positions(), x_mf) < 1e-12
    p.set_operator_memory_limit(0)
    p.set_positions(m.nodes)
    st = p.newton_solve(rel_tol=1e-8, max_newton=30)
    assert st["status"] == 0 and p.operator_info() == (full, False)
    assert rel(p.get_free_positions(), x_as) < 1e-6
