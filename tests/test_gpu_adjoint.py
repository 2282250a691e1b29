"""Adjoint of the static equilibrium behind torch.autograd: gradients with respect to
per-element Young's modulus and dead loads, checked against central finite
differences (h = 1e-4 relative) and against the FP64 oracle's adjoint."""
import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def c5_problem(nx, ny, nz, seed_a=1, seed_b=2):
    from solidfem_gb300.mesh import box_lattice, lumped_face_load

    m = box_lattice(nx, ny, nz, extent=(4.0, 1.0, 1.0))
    fixed = m.face_nodes(0, 0)
    ra, rb = np.random.default_rng(seed_a), np.random.default_rng(seed_b)
    young = 1e5 * np.exp(0.5 * ra.normal(size=m.n_tets))
    young_t = 1e5 * np.exp(0.5 * rb.normal(size=m.n_tets))
    f = lumped_face_load(m, 0, 1, (0.0, 0.0, -1000.0))
    return m, fixed, young, young_t, f


def solve_u(phys, young, f_free, rest, tol=1e-11):
    phys.set_element_youngs(young)
    phys.set_nodal_loads(phys.from_free(f_free))
    phys.set_free_positions(rest)
    st = phys.newton_solve(rel_tol=tol, max_newton=100)
    assert st["status"] == 0, st
    return phys.get_free_positions() - rest


@pytest.mark.parametrize("dims,n_fd", [((16, 4, 4), 8), ((64, 16, 16), 32)])
def test_adjoint_vs_finite_differences_and_oracle(dims, n_fd):
    import torch

    from solidfem_gb300 import FemPhysicsMatrixFree
    from solidfem_gb300.autograd import equilibrium_displacement

    m, fixed, young, young_t, f = c5_problem(*dims)
    phys = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, young=1e5, poisson=0.45, density=1070.0,
                                gravity=(0.0, 0.0, 0.0), material=3)
    rest = phys.rest_free_positions()
    f_free = phys.to_free(f)
    u_t = solve_u(phys, young_t, f_free, rest)
    dev = torch.device("cuda", 0)
    E = torch.tensor(young, device=dev, requires_grad=True)
    F = torch.tensor(f_free, device=dev, requires_grad=True)
    ut = torch.tensor(u_t, device=dev)
    u = equilibrium_displacement(phys, E, F, solve_kw=dict(rel_tol=1e-11, max_newton=100), adjoint_tol=1e-12)
    loss = ((u - ut) ** 2).sum()
    loss.backward()
    gE = E.grad.cpu().numpy()
    gF = F.grad.cpu().numpy()

    def L(yv, fv):
        uu = solve_u(phys, yv, fv, rest)
        return float(((uu - u_t) ** 2).sum())

    rng = np.random.default_rng(3)
    idx = rng.choice(m.n_tets, size=n_fd, replace=False)
    fd = []
    for e in idx:
        h = 1e-4 * young[e]
        yp, ym = young.copy(), young.copy()
        yp[e] += h
        ym[e] -= h
        fd.append((L(yp, f_free) - L(ym, f_free)) / (2 * h))
    fd = np.array(fd)
    scale = np.abs(gE).max()
    err = np.abs(gE[idx] - fd) / scale
    print(f"{dims}: dL/dE vs central FD (h=1e-4 E) on {n_fd} elements: max err / max|g| = {err.max():.2e}")
    assert err.max() < 1e-3
    # directional derivative along a random relative perturbation of all moduli
    v = rng.normal(size=m.n_tets) * young
    hdir = 1e-4
    fdd = (L(young + hdir * v, f_free) - L(young - hdir * v, f_free)) / (2 * hdir)
    assert abs(gE @ v - fdd) <= 1e-5 * abs(fdd), (gE @ v, fdd)
    # load gradient: a few components
    for k in rng.choice(f_free.size, size=4, replace=False):
        i, c = divmod(int(k), 3)
        h = 1e-4 * max(abs(f_free).max(), 1.0)
        fp, fm = f_free.copy(), f_free.copy()
        fp[i, c] += h
        fm[i, c] -= h
        fdv = (L(young, fp) - L(young, fm)) / (2 * h)
        assert abs(gF[i, c] - fdv) <= 1e-4 * np.abs(gF).max() + 1e-6 * abs(fdv)

    # the FP64 oracle's adjoint (the reference gradient): at the oracle's own equilibrium on the small
    # mesh; at the full 98,304-tet size at the GPU's equilibrium, after the oracle's own FP64 residual
    # has certified it (one CPU PCG solve of K lam = dL/du instead of a CPU Newton solve)
    o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, (0.0, 0.0, 0.0), 3)
    o.set_element_scale(young / 1e5)
    o.set_nodal_loads(f)
    if m.n_tets <= 2000:
        status, st_o = o.newton_pcg(rtol=1e-11, max_newton=100)
        assert status == 0, st_o
        uo = o.free_positions().reshape(-1, 3) - rest
    else:
        r0 = np.linalg.norm(o.gradients())
        uo = solve_u(phys, young, f_free, rest)
        o.set_free_positions((rest + uo).ravel())
        r_eq = np.linalg.norm(o.gradients()) / r0
        print(f"{dims}: oracle |r|/|r0| at the GPU equilibrium {r_eq:.2e}")
        assert r_eq <= 1e-9
    dE_o, dF_o, its = o.adjoint((2 * (uo - u_t)).ravel(), young, tol=1e-12, max_cg=200000)
    eE = np.linalg.norm(gE - dE_o) / np.linalg.norm(dE_o)
    eF = np.linalg.norm(gF.ravel() - dF_o) / np.linalg.norm(dF_o)
    print(f"{dims}: adjoint vs the FP64 oracle's ({its} CPU PCG iterations): dL/dE {eE:.2e}, dL/df {eF:.2e}")
    assert eE <= 1e-6 and eF <= 1e-6
