"""Host-side mirror of SolidFEM's FemPhysicsMatrixFree (Include/FemPhysicsMatrixFree.h:43-154)
over the C ABI.  Method names follow the reference class; free-DOF vectors are
(N_f, 3) arrays in the reference's reshuffled order (fixed nodes first).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat


def _dp(a):
    return a.ctypes.data_as(nat._dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class FemPhysicsMatrixFree:
    """GB300 matrix-free nonlinear elasticity for one tetrahedral body.

    Parameters mirror FemConfig (Include/FemDataStructures.h:131-156): ``gravity``
    is either a 3-vector or a scalar applied along z (``zup=True``) or y.
    ``precision`` selects the element kernels / Krylov arithmetic ("fp64" or
    "fp32"; the Newton residual is always FP64).
    """

    def __init__(self, tets, nodes, fixed, young=66000.0, poisson=0.4, density=1070.0, gravity=-9.8,
                 zup=False, material=nat.MMT_NEO_HOOKEAN, precision="fp64", device=0, tangent="reference"):
        self._lib = nat.load()
        nodes = _f64(nodes).reshape(-1, 3)
        tets = np.ascontiguousarray(tets, dtype=np.int32).reshape(-1, 4)
        fixed = np.ascontiguousarray(fixed if fixed is not None else [], dtype=np.int32).ravel()
        g = np.zeros(3)
        if np.ndim(gravity) == 0:
            g[2 if zup else 1] = float(gravity)
        else:
            g[:] = gravity
        cfg = nat.Config()
        cfg.young, cfg.poisson, cfg.density = young, poisson, density
        for c in range(3):
            cfg.gravity[c] = g[c]
        cfg.material = int(material)
        cfg.precision = nat.FP32 if str(precision).lower() in ("fp32", "float32", "1") else nat.FP64
        cfg.device = device
        cfg.tangent = nat.TANGENT_EXACT if tangent in ("exact", 1) else nat.TANGENT_REFERENCE
        h = C.c_void_p()
        nat.check(self._lib.sfem_create(_dp(nodes), nodes.shape[0], tets.ctypes.data_as(nat._ip), tets.shape[0],
                                        fixed.ctypes.data_as(nat._ip), fixed.size, C.byref(cfg), C.byref(h)))
        self._h = h
        self.tets_original, self.rest_positions = tets.copy(), nodes.copy()  # caller's order
        n, nf, e = C.c_int64(), C.c_int64(), C.c_int64()
        self._lib.sfem_sizes(h, C.byref(n), C.byref(nf), C.byref(e))
        self.n_nodes, self.n_free, self.n_tets = n.value, nf.value, e.value
        self.n_bcs = self.n_nodes - self.n_free
        self.young, self.poisson, self.density, self.gravity = young, poisson, density, g
        self.material = int(material)
        self.precision = "fp32" if cfg.precision == nat.FP32 else "fp64"
        self._mu = 0.5 * young / (1 + poisson)
        self._lambda = young * poisson / (1 + poisson) / (1 - 2 * poisson)
        self.device = device
        self._rest_free = None
        self._rest_free = self.get_free_positions()

    # ---- lifetime ----
    def close(self):
        if getattr(self, "_h", None):
            self._lib.sfem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 -- interpreter shutdown
            pass

    @property
    def handle(self):
        return self._h

    # ---- sizes / maps (FemPhysicsMatrixFree.h:74-77) ----
    def GetNumNodes(self):
        return self.n_nodes

    def GetNumFreeNodes(self):
        return self.n_free

    def GetNumElements(self):
        return self.n_tets

    def reshuffle_map(self):
        m = np.zeros(self.n_nodes, dtype=np.int32)
        nat.check(self._lib.sfem_reshuffle_map(self._h, m.ctypes.data_as(nat._ip)))
        return m

    # ---- state ----
    def get_positions(self, out=None):
        """All node positions, original order (N, 3); into ``out`` (float64, C-contiguous (N, 3),
        e.g. a pinned buffer) when given."""
        if out is None:
            out = np.zeros((self.n_nodes, 3))
        elif out.dtype != np.float64 or out.shape != (self.n_nodes, 3) or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of shape (n_nodes, 3)")
        nat.check(self._lib.sfem_get_positions(self._h, _dp(out)))
        return out

    def set_positions(self, pos):
        pos = _f64(pos).reshape(-1, 3)
        nat.check(self._lib.sfem_set_positions(self._h, _dp(pos)))

    def get_free_positions(self):
        x = np.zeros((self.n_free, 3))
        nat.check(self._lib.sfem_get_free_positions(self._h, _dp(x)))
        return x

    def set_free_positions(self, pos):
        pos = _f64(pos).reshape(-1, 3)
        nat.check(self._lib.sfem_set_free_positions(self._h, _dp(pos)))

    def rest_free_positions(self):
        """Free-node rest positions (N_f, 3), reshuffled order."""
        return self._rest_free.copy()

    def to_free(self, a):
        """Original-order node array (N, 3) -> free-node block in reshuffled order (N_f, 3)."""
        a = np.asarray(a, dtype=np.float64).reshape(-1, 3)
        out = np.zeros_like(a)
        out[self.reshuffle_map()] = a
        return out[self.n_bcs:]

    def from_free(self, a_free):
        """Free-node block (N_f, 3) -> original-order array (N, 3), zero at fixed nodes."""
        full = np.zeros((self.n_nodes, 3))
        full[self.n_bcs:] = np.asarray(a_free).reshape(-1, 3)
        return full[self.reshuffle_map()]

    def SetLameParams(self, mu, lam):
        self._mu, self._lambda = mu, lam
        nat.check(self._lib.sfem_set_lame_params(self._h, mu, lam))

    def GetShearModulus(self):
        return self._mu

    def GetLameFirstParam(self):
        return self._lambda

    def set_force_fraction(self, f):
        nat.check(self._lib.sfem_set_force_fraction(self._h, float(f)))

    def set_element_youngs(self, young_e):
        if young_e is None:
            nat.check(self._lib.sfem_set_element_youngs(self._h, None))
        else:
            y = _f64(young_e).ravel()
            assert y.size == self.n_tets
            nat.check(self._lib.sfem_set_element_youngs(self._h, _dp(y)))

    def SetBoundaryConditionsSurface(self, triangles, pressure):
        """Follower pressure on a triangle list of original node indices (FemPhysicsMatrixFree.h:100)."""
        t = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
        self._has_pressure = t.shape[0] > 0
        nat.check(self._lib.sfem_set_pressure_surface(self._h, t.ctypes.data_as(nat._ip), t.shape[0], float(pressure)))

    def set_element_lame(self, mu_e, lambda_e):
        """Per-element Lame parameters (caller's element order); None restores the uniform ones."""
        if mu_e is None:
            nat.check(self._lib.sfem_set_element_lame(self._h, None, None))
            return
        a = _f64(mu_e).ravel()
        b = _f64(lambda_e).ravel()
        assert a.size == b.size == self.n_tets
        nat.check(self._lib.sfem_set_element_lame(self._h, _dp(a), _dp(b)))

    def set_instances(self, node_offsets):
        """Independent bodies: body q owns the nodes [node_offsets[q], node_offsets[q+1])."""
        if node_offsets is None:
            nat.check(self._lib.sfem_set_instances(self._h, 0, None))
            return
        o = np.ascontiguousarray(node_offsets, dtype=np.int64)
        nat.check(self._lib.sfem_set_instances(self._h, o.size - 1, o.ctypes.data_as(nat._i64p)))

    def set_coarse_space(self, cell, rtol=1e-8, modes=6):
        """Two-level learned preconditioner: add the coarse correction P Kc^-1 P^T r of grid-cell
        aggregates of spacing `cell` (rest-state tangent, set up once), P the aggregates' six
        rigid-body modes (modes=6) or twelve affine modes (modes=12); cell <= 0 turns it off."""
        nat.check(self._lib.sfem_set_coarse_space_modes(self._h, float(cell), float(rtol), int(modes)))

    def coarse_apply(self, r):
        """P Kc^-1 P^T r (free DOFs, (N_f, 3))."""
        r = _f64(r).reshape(-1, 3)
        z = np.zeros_like(r)
        nat.check(self._lib.sfem_coarse_apply(self._h, _dp(r), _dp(z)))
        return z

    def coarse_info(self):
        """The coarse space's aggregates, kept modes and setup seconds (rest-state tangent, Kc,
        factorisation + inverse); zeros without one."""
        na, nk = C.c_int32(0), C.c_int32(0)
        secs = np.zeros(3)
        nat.check(self._lib.sfem_coarse_info(self._h, C.byref(na), C.byref(nk), _dp(secs)))
        return {"aggregates": na.value, "coarse_dofs": nk.value, "tangent_s": float(secs[0]),
                "coarse_matrix_s": float(secs[1]), "factorisation_s": float(secs[2])}

    def set_batched_pcg(self, per_instance=True):
        """Krylov solves with instances: every instance's own PCG in one persistent launch (True) or one
        recurrence over all instances (False)."""
        nat.check(self._lib.sfem_set_batched_pcg(self._h, 1 if per_instance else 0))

    def instance_pcg_stats(self, k):
        """Per instance, of the last per-instance PCG solve: (iterations, status, |r|/|b|)."""
        its = np.zeros(k, dtype=np.int32)
        st = np.zeros(k, dtype=np.int32)
        rel = np.zeros(k)
        nat.check(self._lib.sfem_instance_pcg_stats(self._h, its.ctypes.data_as(nat._ip), st.ctypes.data_as(nat._ip),
                                                    _dp(rel)))
        return its, st, rel

    def set_device_wait(self, limit, test=False):
        """Bound (polls) of the persistent kernels' device-side waits; test=True makes the waits run out."""
        nat.check(self._lib.sfem_set_device_wait(self._h, int(limit), 1 if test else 0))

    def instance_stats(self, k):
        rel = np.zeros(k)
        its = np.zeros(k, dtype=np.int32)
        nat.check(self._lib.sfem_instance_stats(self._h, _dp(rel), its.ctypes.data_as(nat._ip)))
        return rel, its

    def set_nodal_loads(self, f):
        """Dead loads (N, 3) in original node order (None clears)."""
        if f is None:
            nat.check(self._lib.sfem_set_nodal_loads(self._h, None))
        else:
            f = _f64(f).reshape(-1, 3)
            nat.check(self._lib.sfem_set_nodal_loads(self._h, _dp(f)))

    # ---- physics (reference member names) ----
    def ComputeGradients(self, return_norm=False):
        r = np.zeros((self.n_free, 3))
        nrm = C.c_double()
        nat.check(self._lib.sfem_compute_gradients(self._h, _dp(r), C.byref(nrm)))
        return (r, nrm.value) if return_norm else r

    def MatrixVectorMultiply(self, d):
        d = _f64(d).reshape(-1, 3)
        out = np.zeros((self.n_free, 3))
        nat.check(self._lib.sfem_matvec(self._h, _dp(d), _dp(out)))
        return out

    def DotProduct(self, a, b):
        a, b = _f64(a), _f64(b)
        out = C.c_double()
        nat.check(self._lib.sfem_dot(self._h, _dp(a), _dp(b), C.byref(out)))
        return out.value

    def UpdatePosAndComputeGradients(self, pos):
        self.set_free_positions(pos)
        return self.ComputeGradients()

    def jacobi_diagonal(self):
        d = np.zeros((self.n_free, 3))
        nat.check(self._lib.sfem_jacobi_diagonal(self._h, _dp(d)))
        return d

    def ComputeElasticEnergy(self):
        e = C.c_double()
        nat.check(self._lib.sfem_energy(self._h, C.byref(e), None))
        return e.value

    def ComputeEnergy(self):
        """Total potential energy (elastic minus work of gravity and dead loads)."""
        t = C.c_double()
        nat.check(self._lib.sfem_energy(self._h, None, C.byref(t)))
        return t.value

    def count_inverted(self):
        n = C.c_int64()
        nat.check(self._lib.sfem_count_inverted(self._h, C.byref(n)))
        return n.value

    def CheckForInversion(self):
        return self.count_inverted() > 0

    def element_stress(self):
        P = np.zeros((self.n_tets, 3, 3))
        nat.check(self._lib.sfem_element_stress(self._h, _dp(P)))
        return P

    def GetForceParamGrads(self):
        a, b, c = (np.zeros((self.n_free, 3)) for _ in range(3))
        nat.check(self._lib.sfem_force_param_grads(self._h, _dp(a), _dp(b), _dp(c)))
        return a.ravel(), b.ravel(), c.ravel()

    # ---- solvers ----
    def pcg(self, b, rel_tol=1e-8, max_iters=10000, precond=nat.PC_JACOBI):
        b = _f64(b).reshape(-1, 3)
        x = np.zeros_like(b)
        o = nat.PcgOpts(rel_tol=rel_tol, max_iters=max_iters, precond=precond, check_every=0)
        st = nat.PcgStats()
        code = nat.check(self._lib.sfem_pcg(self._h, _dp(b), _dp(x), C.byref(o), C.byref(st)))
        return x, dict(iters=st.iters, rel_res=st.rel_res, status=code)

    def newton_solve(self, rel_tol=1e-8, abs_tol=0.0, max_newton=50, max_cg=100000, precond=nat.PC_JACOBI,
                     ls_condition=None, eta_max=0.5, eta_min=0.0, load_steps=1, verbose=False,
                     max_bisection=0):
        """Globalised inexact Newton.  The default line search is energy Armijo for the
        hyperelastic materials and residual-norm backtracking for corotational (whose force
        is not the gradient of an energy)."""
        if ls_condition is None:
            nonconservative = (self.material == nat.MMT_COROTATIONAL or getattr(self, "_has_pressure", False)
                               or self.material not in nat.MATERIALS_WITH_ENERGY)
            ls_condition = nat.LSC_RESIDUAL if nonconservative else nat.LSC_ARMIJO
        o = nat.NewtonOpts(rel_tol=rel_tol, abs_tol=abs_tol, max_newton=max_newton, max_cg=max_cg, eta_max=eta_max,
                           eta_min=eta_min, precond=precond, ls_condition=ls_condition,
                           max_bisection=max_bisection, verbose=int(verbose), load_steps=load_steps)
        st = nat.NewtonStats()
        code = nat.check(self._lib.sfem_newton_solve(self._h, C.byref(o), C.byref(st)))
        return dict(status=code, newton_iters=st.newton_iters, cg_iters=st.cg_iters, r0=st.r0,
                    rel_res=st.rel_res, seconds=st.seconds, line_search_cuts=st.line_search_cuts)

    def Step(self, dt=0.0, simtype=0, substeps=1, **newton_kw):
        """FemPhysicsMatrixFree::Step (Source/FemPhysicsMatrixFree.cpp:297-342): static
        (simtype 0/1: the Newton solve), explicit (2: symplectic Euler substeps on the elastic
        forces and gravity) or implicit (3: backward Euler, a Newton solve per substep)."""
        if simtype in (0, 1) or dt == 0:
            return self.newton_solve(**newton_kw)
        if simtype == nat.SIM_EXPLICIT:
            nat.check(self._lib.sfem_step(self._h, float(dt), nat.SIM_EXPLICIT, int(substeps), None, None))
            return dict(status=0)
        kw = dict(rel_tol=1e-8, abs_tol=0.0, max_newton=50, max_cg=100000, precond=nat.PC_JACOBI,
                  ls_condition=nat.LSC_ARMIJO if (self.material in nat.MATERIALS_WITH_ENERGY
                                                  and self.material != nat.MMT_COROTATIONAL) else nat.LSC_RESIDUAL,
                  eta_max=0.5, eta_min=0.0, load_steps=1, verbose=0, max_bisection=0)
        kw.update(newton_kw)
        o = nat.NewtonOpts(**kw)
        st = nat.NewtonStats()
        code = nat.check(self._lib.sfem_step(self._h, float(dt), nat.SIM_IMPLICIT, int(substeps), C.byref(o),
                                             C.byref(st)))
        return dict(status=code, newton_iters=st.newton_iters, cg_iters=st.cg_iters, r0=st.r0, rel_res=st.rel_res,
                    seconds=st.seconds, line_search_cuts=st.line_search_cuts)

    def set_time_step(self, dt):
        """mTimeStep: 0 for static, h > 0 adds the backward-Euler inertia terms."""
        nat.check(self._lib.sfem_set_time_step(self._h, float(dt)))

    def set_velocities(self, vel):
        v = _f64(vel).reshape(-1, 3)
        nat.check(self._lib.sfem_set_velocities(self._h, _dp(v)))

    def get_velocities(self):
        v = np.zeros((self.n_nodes, 3))
        nat.check(self._lib.sfem_get_velocities(self._h, _dp(v)))
        return v

    def begin_step(self):
        """x_start = x (the reference's pos0 = pos at the start of an implicit Step)."""
        nat.check(self._lib.sfem_begin_step(self._h))

    def set_newton_trace(self, cap=100000):
        """Record every line-search trial of the following Newton solves (cap trials; 0 stops it):
        newton_trace() then returns rows (Newton iteration, step length, |r| at the trial)."""
        if cap <= 0:
            nat.check(self._lib.sfem_set_newton_trace(self._h, None, 0, None))
            self._trace = None
            return
        buf = np.zeros((cap, 3))
        cnt = C.c_int32(0)
        nat.check(self._lib.sfem_set_newton_trace(self._h, _dp(buf), cap, C.byref(cnt)))
        self._trace = (buf, cnt)  # kept alive while the library writes into them

    def newton_trace(self):
        buf, cnt = self._trace
        return buf[:cnt.value].copy()

    def nonlinear_cg(self, outer_iters=200, inner_iters=10, abs_tol=1e-4):
        it = C.c_int32()
        nat.check(self._lib.sfem_nonlinear_cg(self._h, outer_iters, inner_iters, abs_tol, C.byref(it)))
        return it.value

    def adjoint(self, dLdu, rel_tol=1e-10, max_cg=100000):
        """Gradients of L at equilibrium: (dL/dE_e (E,), dL/df_ext (N_f, 3))."""
        g = _f64(dLdu).reshape(-1, 3)
        dE = np.zeros(self.n_tets)
        df = np.zeros((self.n_free, 3))
        nat.check(self._lib.sfem_adjoint(self._h, _dp(g), rel_tol, max_cg, _dp(dE), _dp(df)))
        return dE, df

    def set_operator(self, op: str) -> None:
        """Operator of the Krylov solves: 'matrix-free' (the patch product, default) or 'assembled'
        (the tangent assembled in the handle's precision at every Newton step, one sparse product
        per iteration; materials 0-3, single bodies)."""
        nat.check(self._lib.sfem_set_operator(self._h, {"matrix-free": nat.OP_MATRIX_FREE,
                                                         "assembled": nat.OP_ASSEMBLED}[op]))

    def set_residual_arithmetic(self, mode: str) -> None:
        """Arithmetic of the nonlinear residual's element pass for FP32 neo-Hookean handles: 'two-term'
        (default: two-term FP32, FP64-accurate, on the FP32 pipes) or 'fp64' (FP64 instructions).  FP64
        handles and the other materials always use FP64."""
        nat.check(self._lib.sfem_set_residual_arithmetic(self._h, {"fp64": nat.RESIDUAL_FP64,
                                                                    "two-term": nat.RESIDUAL_TWO_TERM}[mode]))

    def set_operator_memory_limit(self, nbytes: int) -> None:
        """Cap on the device memory of the assembled operator (0: none); beyond it the Krylov solves
        keep the matrix-free product."""
        nat.check(self._lib.sfem_set_operator_memory_limit(self._h, int(nbytes)))

    def operator_info(self):
        """(bytes held by the assembled operator, True when its assembly ran out of memory)."""
        b = C.c_int64()
        f = C.c_int32()
        nat.check(self._lib.sfem_operator_info(self._h, C.byref(b), C.byref(f)))
        return b.value, bool(f.value)

    def set_profiling(self, enable=True):
        nat.check(self._lib.sfem_set_profiling(self._h, int(enable)))

    def get_profile(self):
        pr = nat.Profile()
        nat.check(self._lib.sfem_get_profile(self._h, C.byref(pr)))
        return {k: getattr(pr, k) for k, _ in nat.Profile._fields_ if k != "reserved"}

    @staticmethod
    def kernel_launches():
        n = C.c_int64()
        nat.check(nat.load().sfem_kernel_launches(C.byref(n)))
        return n.value

    def get_hessian_sparse(self):
        """The assembled FP64 tangent over free DOFs (reshuffled order) as a scipy BSR matrix with
        3 x 3 blocks (ElasticEnergy::AssembleStiffnessMatrix, assembled on the GPU)."""
        import scipy.sparse as sp

        nnzb = C.c_int64()
        nat.check(self._lib.sfem_tangent_nnz(self._h, C.byref(nnzb)))
        rowptr = np.zeros(self.n_free + 1, dtype=np.int32)
        col = np.zeros(nnzb.value, dtype=np.int32)
        vals = np.zeros((nnzb.value, 3, 3))
        nat.check(self._lib.sfem_assemble_tangent(self._h, rowptr.ctypes.data_as(nat._ip),
                                                  col.ctypes.data_as(nat._ip), _dp(vals)))
        n = 3 * self.n_free
        return sp.bsr_matrix((vals, col, rowptr), shape=(n, n))

    def get_hessian(self):
        """Dense tangent over free DOFs (what pysolidfem's get_hessian returns), from the GPU assembly."""
        return self.get_hessian_sparse().toarray()

    def tangent_matvec(self, d):
        d = _f64(d).ravel()
        out = np.zeros_like(d)
        nat.check(self._lib.sfem_tangent_matvec(self._h, _dp(d), _dp(out)))
        return out
