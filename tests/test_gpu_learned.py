"""Learned preconditioner on the GPU: forward and gradients of the hand-written BF16
tensor-core kernels against the FP64 oracle (oracle/gnn_oracle.py), and what the trained
network gains over Jacobi inside the Newton-Krylov solve, held to the same FP64
residual tolerance."""
import numpy as np
import pytest

from oracle import gnn_oracle as go
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def slab(nx, ny, nz, seed_load=0):
    from solidfem_gb300.mesh import box_lattice, random_top_traction

    m = box_lattice(nx, ny, nz, extent=(4.0 * nx / 256, 1.0 * ny / 64, 1.0 * nz / 64), jitter=0.2, seed=0)
    fixed = m.face_nodes(2, 0)
    return m, fixed, random_top_traction(m, seed=seed_load)


def gpu_and_oracle(m, fixed, seed=0):
    from solidfem_gb300 import FemPhysicsMatrixFree
    from solidfem_gb300.learned import LearnedPreconditioner

    p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, young=1e5, poisson=0.49, density=1070.0, gravity=(0, 0, 0),
                             material=3, precision="fp32")
    net = LearnedPreconditioner(p, seed=seed)
    o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.49, 1070.0, (0, 0, 0), 3)
    Am = go.free_graph(o.tets(), o.n_bcs, o.n_nodes)
    dinv = 1.0 / o.jacobi_diagonal()
    return p, net, o, Am, dinv


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


@pytest.mark.parametrize("mode", ["poly", "layers"])
def test_forward_matches_fp64_oracle(mode):
    m, fixed, _ = slab(24, 8, 8)
    p, net, o, Am, dinv = gpu_and_oracle(m, fixed, seed=3)
    net.set_inference(mode)
    rng = np.random.default_rng(1)
    r = rng.normal(size=3 * o.n_free)
    out_g = net.apply(r)
    out_o = go.forward(net.get_params(), Am, r, dinv)
    err = rel(out_g, out_o)
    # the S^T S part alone (c x removed), where the BF16 rounding lives
    prm = net.get_params().astype(np.float64)
    c = np.exp(prm[go.OFF_C])
    ss_g, ss_o = out_g - c * dinv * r, out_o - c * dinv * r
    err_ss = rel(ss_g, ss_o)
    print(f"M(r) GPU ({mode}) vs FP64 oracle: rel err {err:.2e}; S^T S part {err_ss:.2e}; {net.graph_form()}")
    assert err < 2e-2 and err_ss < 3e-2
    if mode == "poly":  # FP32 arithmetic on the folded coefficients over FP16 node rows (11-bit
        # significand, scaled into range): about 3.5e-4 here in a numpy model of the same rounding
        assert err_ss < 2e-3
        # a lattice's free nodes fall in 3 x 3 x 3 neighbour patterns (interior, faces, edges,
        # corners; the layer above the clamped face is a class of its own)
        assert net.graph_form()[0] == "patterns"
        assert net.graph_form()[1] == 27
    # linear and symmetric on the device too (up to BF16 rounding of the activations)
    u, v = rng.normal(size=(2, 3 * o.n_free))
    Mu, Mv = net.apply(u), net.apply(v)
    assert abs(u @ Mv - v @ Mu) <= 2e-2 * abs(u @ Mv)
    assert rel(net.apply(2.0 * u + v), 2.0 * Mu + Mv) < 2e-2


def test_forward_without_shared_patterns():
    """The polynomial passes on a randomly numbered mesh, where no two nodes share a neighbour
    list: the per-node 16-bit deltas are read instead of the pattern table."""
    m, fixed, _ = slab(24, 8, 8)
    perm = np.random.default_rng(5).permutation(len(m.nodes))
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm))
    m.nodes = m.nodes[perm]
    m.tets = inv[m.tets].astype(np.int32)
    fixed = inv[fixed]
    p, net, o, Am, dinv = gpu_and_oracle(m, fixed, seed=3)
    assert net.graph_form()[0] == "delta16"
    r = np.random.default_rng(1).normal(size=3 * o.n_free)
    out_g = net.apply(r)
    out_o = go.forward(net.get_params(), Am, r, dinv)
    c = np.exp(net.get_params().astype(np.float64)[go.OFF_C])
    err_ss = rel(out_g - c * dinv * r, out_o - c * dinv * r)
    print(f"M(r) GPU (poly, per-node deltas) vs FP64 oracle: S^T S part {err_ss:.2e}")
    assert err_ss < 2e-3  # FP16 node rows, as above


@pytest.mark.parametrize("mode", ["energy", "residual"])
def test_gradients_match_fp64_oracle(mode):
    m, fixed, _ = slab(24, 8, 8)
    p, net, o, Am, dinv = gpu_and_oracle(m, fixed, seed=4)
    rng = np.random.default_rng(2)
    r = rng.normal(size=3 * o.n_free)
    e, _, _ = o.pcg(r, diag=1.0 / dinv, tol=1e-10, max_iters=20000)
    net.set_loss(mode)
    Lg, gg = net.loss_grad(r, e)
    Lo, go_ = go.loss_grad(net.get_params(), Am, r, dinv, e, o.matvec, mode=mode)
    cos = float(gg @ go_) / (np.linalg.norm(gg) * np.linalg.norm(go_))
    print(f"loss GPU {Lg:.6f} oracle {Lo:.6f}; grad rel err {rel(gg, go_):.2e}, cosine {cos:.5f}")
    assert abs(Lg - Lo) <= 3e-2 * abs(Lo)
    assert rel(gg, go_) < 8e-2 and cos > 0.995
    for name, a, b in [("We", go.OFF_WE, go.OFF_L), ("L1", go.OFF_L, go.OFF_L + go.L_STRIDE),
                       ("L3", go.OFF_L + 2 * go.L_STRIDE, go.OFF_C), ("log c", go.OFF_C, go.NPARAM)]:
        assert rel(gg[a:b], go_[a:b]) < 1e-1, name


def test_trained_network_gain_over_jacobi():
    """Train on residual/correction pairs from plain solves of small slabs (load seeds 0..15),
    evaluate on a held-out load (seed 10000): iterations and time of the learned flexible PCG
    against Jacobi-PCG, both to the same 1e-8 FP64 residual."""
    from solidfem_gb300 import FemPhysicsMatrixFree, PC_JACOBI, PC_LEARNED
    from solidfem_gb300.learned import LearnedPreconditioner

    m, fixed, _ = slab(64, 16, 16)
    kw = dict(young=1e5, poisson=0.49, density=1070.0, gravity=(0, 0, 0), material=3, precision="fp32")
    p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, **kw)
    net = LearnedPreconditioner(p, seed=0)
    from solidfem_gb300.mesh import random_top_traction

    for s in range(16):
        p.set_nodal_loads(random_top_traction(m, seed=s))
        net.collect(None, every=25, max_snaps=40, rel_tol=1e-6)
    n = net.dataset_size()
    net.set_batch(8)
    losses = net.train(steps=600, lr=1e-3, seed=0)
    first, last = float(np.mean(losses[:50])), float(np.mean(losses[-50:]))
    print(f"pairs {n}; energy-norm loss {first:.4f} -> {last:.4f}")
    assert last < first
    f_eval = random_top_traction(m, seed=10000)
    res = {}
    for name, pc in [("jacobi", PC_JACOBI), ("learned", PC_LEARNED), ("learned-layers", PC_LEARNED)]:
        if name == "learned-layers":
            net.set_inference("layers")
        p.set_nodal_loads(f_eval)
        p.set_positions(m.nodes)
        st = p.newton_solve(rel_tol=1e-8, max_newton=30, precond=pc)
        assert st["status"] == 0 and st["rel_res"] <= 1e-8, (name, st)
        res[name] = st
    print("jacobi:", res["jacobi"], "\nlearned:", res["learned"], "\nlearned, layer kernels:", res["learned-layers"])
    ratio = res["learned"]["cg_iters"] / res["jacobi"]["cg_iters"]
    print(f"learned/jacobi CG iterations {ratio:.3f}, time {res['learned']['seconds'] / res['jacobi']['seconds']:.3f}")
    assert ratio < 0.7
