"""Drop-in for the reference's Python module ``pysolidfem`` (PySolidFEM/Module.cpp:90-112,
PySolidFEM/PyNonlinearFEM.cpp) for the matrix-free static path.

``NonlinearFEM(tets, nodes, fixed_nodes, config)`` accepts the reference's config
keys (young, poisson, density, simtype, substeps, maxiter, tol, mixed,
optimizer; PyNonlinearFEM::ParseConfig, PyNonlinearFEM.cpp:240-293) and a
backward-compatible superset: material, solver, gravity, zup, precision,
precond, cg_tol, newton_rtol.  As in the reference, the material defaults to
neo-Hookean and gravity to -9.8 along y.
"""
from __future__ import annotations

import numpy as np

from . import _native as nat
from .physics import FemPhysicsMatrixFree

# SimulationType (Include/FemDataStructures.h:71-77)
ST_STATIC, ST_QUASI_STATIC, ST_EXPLICIT, ST_IMPLICIT = 0, 1, 2, 3
# NonlinearSolverType (Include/FemDataStructures.h:107-120)
NST_NEWTON, NST_NEWTON_LS, NST_NEWTON_CG, NST_NONLINEAR_CG = 0, 1, 2, 3

_MATERIALS = {"linear": nat.MMT_LINEAR, "stvk": nat.MMT_STVK, "corotational": nat.MMT_COROTATIONAL,
              "neo-hookean": nat.MMT_NEO_HOOKEAN, "neohookean": nat.MMT_NEO_HOOKEAN,
              "neo-hookean-ogden": nat.MMT_NEO_HOOKEAN_OGDEN, "distortional-linear": nat.MMT_DISTORTIONAL_LINEAR,
              "distortional-mooney": nat.MMT_DISTORTIONAL_MOONEY, "distortional-nh2": nat.MMT_DISTORTIONAL_NH2,
              "distortional-nh3": nat.MMT_DISTORTIONAL_NH3, "distortional-bw": nat.MMT_DISTORTIONAL_BW,
              "distortional-ogden": nat.MMT_DISTORTIONAL_OGDEN, "distortional-nh6": nat.MMT_DISTORTIONAL_NH6,
              "distortional-nh7": nat.MMT_DISTORTIONAL_NH7}


class NonlinearFEM:
    def __init__(self, tets, nodes, fixed_nodes, config=None):
        cfg = dict(config or {})
        if cfg.get("mixed", False):
            raise NotImplementedError("mixed FEM (FemPhysicsMixed) is outside the matrix-free path")
        tets = np.asarray(tets, dtype=np.int32)
        if tets.ndim == 1 or tets.shape[-1] != 4:  # the reference accepts a flat index list
            tets = tets.reshape(-1, 4)
        nodes = np.asarray(nodes, dtype=np.float64)
        if nodes.ndim != 2 or nodes.shape[1] != 3:
            raise ValueError("Nodes should have 3 columns")
        mat = cfg.get("material", nat.MMT_NEO_HOOKEAN)
        if isinstance(mat, str):
            mat = _MATERIALS[mat.lower()]
        gravity = cfg.get("gravity", -9.8)
        self.simtype = int(cfg.get("simtype", ST_STATIC))
        self.substeps = int(cfg.get("substeps", 1))
        self.maxiter = int(cfg.get("maxiter", 10))  # FemConfig::mOuterIterations default
        self.tol = float(cfg.get("tol", 0.1))  # FemConfig::mAbsNewtonRsidualThreshold default
        self.optimizer = bool(cfg.get("optimizer", False))
        self.solver = int(cfg.get("solver", NST_NEWTON_LS))
        self.precond = int(cfg.get("precond", nat.PC_JACOBI))
        self.newton_rtol = float(cfg.get("newton_rtol", 0.0))
        self.force_step = float(cfg.get("force_step", 0.1))  # FemConfig::mForceApplicationStep
        self.phys = FemPhysicsMatrixFree(tets, nodes, fixed_nodes, young=float(cfg.get("young", 66000.0)),
                                         poisson=float(cfg.get("poisson", 0.4)),
                                         density=float(cfg.get("density", 1070.0)), gravity=gravity,
                                         zup=bool(cfg.get("zup", False)), material=mat,
                                         precision=cfg.get("precision", "fp64"))
        self._tets = tets
        self.force_fraction = 0.0
        self._grads = None
        self.last_stats = None

    # PyNonlinearFEM::Step (PyNonlinearFEM.cpp:126-132) -> FemPhysicsMatrixFree::Step (:297-342)
    def step(self, dt=0.016):
        if self.simtype == ST_STATIC:
            if self.force_fraction == 0:
                self.force_fraction = 1.0
                self._solve()
        elif self.simtype == ST_QUASI_STATIC:
            if self.force_fraction < 1:
                self.force_fraction = min(1.0, self.force_fraction + self.force_step)
                self._solve()
        elif self.simtype == ST_EXPLICIT:
            self.phys.Step(dt, simtype=ST_EXPLICIT, substeps=self.substeps)
        elif self.simtype == ST_IMPLICIT:
            self.force_fraction = 1.0
            self.phys.set_force_fraction(1.0)
            lsc = nat.LSC_ARMIJO if self.optimizer else nat.LSC_ENGINEERING
            self.last_stats = self.phys.Step(dt, simtype=ST_IMPLICIT, substeps=self.substeps, rel_tol=self.newton_rtol,
                                             abs_tol=self.tol, max_newton=self.maxiter, precond=self.precond,
                                             ls_condition=lsc, eta_min=1e-10)

    def simulate_static(self):
        while self.force_fraction < 1:
            self.simtype = ST_QUASI_STATIC if self.simtype == ST_QUASI_STATIC else self.simtype
            prev = self.force_fraction
            self.step(0)
            if self.force_fraction == prev:
                break

    def _solve(self):
        self.phys.set_force_fraction(self.force_fraction)
        if self.solver == NST_NONLINEAR_CG:
            self.phys.nonlinear_cg(outer_iters=self.maxiter, inner_iters=100, abs_tol=self.tol)
            return
        lsc = nat.LSC_ARMIJO if self.optimizer else nat.LSC_ENGINEERING
        if self.solver == NST_NEWTON_CG:
            lsc = nat.LSC_RESIDUAL
        self.last_stats = self.phys.newton_solve(rel_tol=self.newton_rtol, abs_tol=self.tol,
                                                 max_newton=self.maxiter, precond=self.precond,
                                                 ls_condition=lsc, eta_min=1e-10)

    def get_nodes(self):
        return self.phys.get_positions()

    def get_tets(self):
        return self._tets.copy()

    def set_lame_params(self, mu, lam):
        self.phys.SetLameParams(mu, lam)

    def get_shear_modulus(self):
        return self.phys.GetShearModulus()

    def get_lame_lambda(self):
        return self.phys.GetLameFirstParam()

    def get_hessian(self):
        return self.phys.get_hessian()

    def compute_force_param_grads(self):
        self._grads = self.phys.GetForceParamGrads()

    def get_force_mu_grad(self):
        return self._grads[0]

    def get_force_lambda_grad(self):
        return self._grads[1]

    def get_force_rho_grad(self):
        # the reference returns the lambda gradient here (PyNonlinearFEM.h:71); this returns d f / d rho
        return self._grads[2]
