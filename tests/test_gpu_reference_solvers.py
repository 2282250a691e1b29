"""The reference's own nonlinear solvers, reproduced through the C ABI on the C1 cantilever
(16x4x4 hexes x 6 tets, neo-Hookean, nu = 0.45, gravity -9.81 z, x = 0 clamped), against
fixtures the reference produced (tests/golden/make_golden.py, reference_solvers):

* NonlinearConjugateGradientMinimizer::Solve (Include/NonlinearCG.h:51-114): the iterate after
  k outer iterations (10 inner Newton-Raphson line-search steps) equals the reference's.
* NewtonSolverBackTrack::Solve with the Bonet-Wood condition (Include/NewtonSolver.h:179-348, the
  default of FemPhysicsMatrixFree::SolveNewtonLS, Source/FemPhysicsMatrixFree.cpp:733-781): with
  the inner linear solves tight (the reference factorises the tangent), every line-search trial
  -- its Newton iteration, its step length on the bisection and its residual norm -- matches the
  reference's while the bisection's decisions are above rounding, and the solution matches.  The
  condition as coded, Rnew < 0.5 Rold with Rold = -delta.r < 0, accepts only steps below 1/2 where
  the residual is nearly linear in the step, so from about |r| = 1e-12 |r0| on every accepted step
  sits within 2^-23 of 1/2 and rounding decides the bisection (the reference's own run then wanders
  at |r| ~ 2e-13 |r0| for twenty more iterations)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _handle(g, young):
    from solidfem_gb300 import FemPhysicsMatrixFree

    return FemPhysicsMatrixFree(g["tets"], g["nodes"], g["fixed"], young=float(young), poisson=float(g["poisson"]),
                                density=float(g["density"]), gravity=tuple(g["gravity"]), material=int(g["material"]),
                                precision="fp64")


def test_nonlinear_cg_iterates_match_reference(golden):
    g = golden("nlcg_c1.npz")
    for young, k, ref_pos in zip(g["young"], g["outer_iters"], g["positions"]):
        p = _handle(g, young)
        p.nonlinear_cg(outer_iters=int(k), inner_iters=int(g["inner_iters"]), abs_tol=float(g["abs_tol"]))
        x = p.get_positions()
        err = np.linalg.norm(x - ref_pos) / np.linalg.norm(ref_pos - g["nodes"])
        print(f"NLCG E={young:g} after {k} outer iterations: displacement error vs the reference {err:.2e}")
        assert err <= 1e-10, (young, k, err)
        p.close()


def test_bonet_wood_line_search_matches_reference_trial_by_trial(golden):
    from solidfem_gb300 import LSC_ENGINEERING, PC_JACOBI

    g = golden("bw_c1.npz")
    p = _handle(g, g["young"])
    p.set_newton_trace(20000)
    st = p.newton_solve(rel_tol=1e-300, abs_tol=float(g["abs_tol"]), max_newton=400, max_cg=200000,
                        precond=PC_JACOBI, ls_condition=LSC_ENGINEERING, eta_max=1e-12, eta_min=1e-12)
    tr = p.newton_trace()
    p.set_newton_trace(0)
    it, step, res = g["trial_iter"], g["trial_step"], g["trial_res"]
    r0 = float(g["r0"])
    print(f"Bonet-Wood: GPU {st['newton_iters']} Newton iterations, {len(tr)} trials; reference "
          f"{it.max() + 1} iterations, {it.size} trials")
    # the leading iterations whose trials all stay above 1e-12 |r0|: decided above rounding
    decisive = 0
    while decisive <= it.max() and res[it == decisive].min() >= 1e-12 * r0:
        decisive += 1
    n = int((it < decisive).sum())
    print(f"trial-by-trial over the first {decisive} iterations ({n} trials)")
    assert decisive >= 30 and len(tr) >= n
    for k in range(n):
        same = (int(tr[k, 0]) == it[k] and abs(tr[k, 1] - step[k]) <= 1e-9
                and abs(tr[k, 2] - res[k]) <= 1e-7 * res[k] + 1e-12 * r0)
        assert same, (f"trial {k}: GPU (iteration {int(tr[k, 0])}, step {tr[k, 1]!r}, |r| {tr[k, 2]:.9e}) vs "
                      f"reference (iteration {it[k]}, step {step[k]!r}, |r| {res[k]:.9e})")
    assert st["status"] == 0
    x = p.get_positions()
    err = np.linalg.norm(x - g["eq_positions"]) / np.linalg.norm(g["eq_positions"] - g["nodes"])
    print(f"solution vs the reference's: {err:.2e}")
    assert err <= 1e-9
