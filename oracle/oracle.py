"""TEST INFRASTRUCTURE ONLY: ctypes wrappers for the oracle (sfem_oracle.c) and,
where the reference tree is present, the reference harness (oracle/_ref).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsfem_ref.so")
# the reference source tree (present in the development container only); SFEM_REF_TREE overrides it
REF_TREE = os.environ.get("SFEM_REF_TREE", "/root/reference")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

MMT_LINEAR, MMT_STVK, MMT_COROTATIONAL, MMT_NEO_HOOKEAN = 0, 1, 2, 3


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "sfem_oracle.c")
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-std=c99", "-O2", "-fopenmp", "-fPIC", "-ffp-contract=off",
                               "-shared", "-o", ORACLE_SO, src, "-lm"])
    return ORACLE_SO


def build_ref() -> str | None:
    """Compile the reference hot path + harness (only where the reference exists)."""
    if not os.path.isdir(REF_TREE):
        return None
    root = os.path.dirname(HERE)
    subprocess.check_call(["make", "-s", "-j8", "-f", "oracle/Makefile.ref", f"REF={REF_TREE}"], cwd=root)
    return REF_SO


def _p(a, ctype=_dp):
    return a.ctypes.data_as(ctype)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Oracle:
    """The C restatement of the reference matrix-free physics (FP64 CPU)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = C.CDLL(build_oracle())
            lib.orc_create.restype = C.c_void_p
            lib.orc_create.argtypes = [_dp, C.c_int, _ip, C.c_int, _ip, C.c_int, C.c_double, C.c_double,
                                       C.c_double, _dp, C.c_int]
            for name in ["orc_destroy"]:
                getattr(lib, name).argtypes = [C.c_void_p]
            for name in ["orc_num_bcs", "orc_num_free", "orc_count_inverted"]:
                getattr(lib, name).argtypes = [C.c_void_p]
                getattr(lib, name).restype = C.c_int
            for name in ["orc_reshuffle_map", "orc_tets"]:
                getattr(lib, name).argtypes = [C.c_void_p, _ip]
            for name in ["orc_set_nodal_loads", "orc_set_positions_shuffled", "orc_get_positions_shuffled",
                         "orc_get_positions", "orc_set_free_positions", "orc_get_free_positions",
                         "orc_compute_gradients", "orc_jacobi_diagonal", "orc_element_stress",
                         "orc_element_forces", "orc_set_element_scale"]:
                getattr(lib, name).argtypes = [C.c_void_p, _dp]
            lib.orc_set_force_fraction.argtypes = [C.c_void_p, C.c_double]
            lib.orc_set_time_step.argtypes = [C.c_void_p, C.c_double]
            lib.orc_explicit_substep.argtypes = [C.c_void_p, C.c_double]
            for name in ["orc_set_velocities_shuffled", "orc_get_velocities_shuffled", "orc_set_start_shuffled"]:
                getattr(lib, name).argtypes = [C.c_void_p, _dp]
            lib.orc_set_lame.argtypes = [C.c_void_p, C.c_double, C.c_double]
            lib.orc_set_tangent.argtypes = [C.c_void_p, C.c_int]
            lib.orc_set_pressure_surface.argtypes = [C.c_void_p, _ip, C.c_int, C.c_double]
            lib.orc_matvec.argtypes = [C.c_void_p, _dp, _dp]
            for name in ["orc_elastic_energy", "orc_total_energy"]:
                getattr(lib, name).argtypes = [C.c_void_p]
                getattr(lib, name).restype = C.c_double
            lib.orc_force_param_grads.argtypes = [C.c_void_p, _dp, _dp, _dp]
            lib.orc_pcg.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_double, C.c_int, _dp]
            lib.orc_pcg.restype = C.c_int
            lib.orc_newton_pcg.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double, _dp]
            lib.orc_newton_pcg.restype = C.c_int
            lib.orc_adjoint.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int, _dp, _dp]
            lib.orc_adjoint.restype = C.c_int
            lib.orc_num_threads.restype = C.c_int
            cls._lib = lib
        return cls._lib

    def __init__(self, nodes, tets, fixed, young, poisson, density=1070.0, gravity=(0.0, 0.0, 0.0),
                 material=MMT_NEO_HOOKEAN):
        lib = self.lib()
        self.nodes = _f64(nodes)
        self.tets_in = _i32(tets)
        self.fixed = _i32(fixed)
        g = _f64(gravity)
        self.n_nodes = self.nodes.shape[0]
        self.n_tets = self.tets_in.shape[0]
        self.h = lib.orc_create(_p(self.nodes), self.n_nodes, _p(self.tets_in, _ip), self.n_tets,
                                _p(self.fixed, _ip), self.fixed.size, young, poisson, density, _p(g), material)
        self.n_bcs = lib.orc_num_bcs(self.h)
        self.n_free = lib.orc_num_free(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib().orc_destroy(self.h)
            self.h = None

    def _vec(self, n):
        return np.zeros(n, dtype=np.float64)

    def reshuffle_map(self):
        m = np.zeros(self.n_nodes, dtype=np.int32)
        self.lib().orc_reshuffle_map(self.h, _p(m, _ip))
        return m

    def tets(self):
        t = np.zeros((self.n_tets, 4), dtype=np.int32)
        self.lib().orc_tets(self.h, _p(t, _ip))
        return t

    def set_force_fraction(self, f):
        self.lib().orc_set_force_fraction(self.h, f)

    # ---- dynamics (reshuffled node order) ----
    def set_time_step(self, dt):
        self.lib().orc_set_time_step(self.h, float(dt))

    def set_velocities_shuffled(self, v):
        v = _f64(v).reshape(-1, 3)
        self.lib().orc_set_velocities_shuffled(self.h, _p(v))

    def velocities_shuffled(self):
        v = np.zeros((self.n_nodes, 3))
        self.lib().orc_get_velocities_shuffled(self.h, _p(v))
        return v

    def set_start_shuffled(self, x):
        x = _f64(x).reshape(-1, 3)
        self.lib().orc_set_start_shuffled(self.h, _p(x))

    def explicit_substep(self, hs):
        self.lib().orc_explicit_substep(self.h, float(hs))

    def set_lame(self, mu, lam):
        self.lib().orc_set_lame(self.h, mu, lam)

    def set_tangent(self, mode):
        self.lib().orc_set_tangent(self.h, mode)

    def set_pressure_surface(self, tris, pressure):
        self._tris = _i32(tris)
        self.lib().orc_set_pressure_surface(self.h, _p(self._tris, _ip), self._tris.shape[0], pressure)

    def set_element_scale(self, s):
        if s is None:
            self.lib().orc_set_element_scale(self.h, None)
        else:
            self._escale = _f64(s)
            self.lib().orc_set_element_scale(self.h, _p(self._escale))

    def set_nodal_loads(self, f):
        f = _f64(f)
        self.lib().orc_set_nodal_loads(self.h, _p(f))

    def set_positions_shuffled(self, x):
        x = _f64(x)
        self.lib().orc_set_positions_shuffled(self.h, _p(x))

    def positions_shuffled(self):
        x = self._vec(3 * self.n_nodes)
        self.lib().orc_get_positions_shuffled(self.h, _p(x))
        return x.reshape(-1, 3)

    def positions(self):
        x = self._vec(3 * self.n_nodes)
        self.lib().orc_get_positions(self.h, _p(x))
        return x.reshape(-1, 3)

    def set_free_positions(self, x):
        x = _f64(x)
        self.lib().orc_set_free_positions(self.h, _p(x))

    def free_positions(self):
        x = self._vec(3 * self.n_free)
        self.lib().orc_get_free_positions(self.h, _p(x))
        return x

    def gradients(self):
        r = self._vec(3 * self.n_free)
        self.lib().orc_compute_gradients(self.h, _p(r))
        return r

    def matvec(self, d):
        d = _f64(d).ravel()
        out = self._vec(3 * self.n_free)
        self.lib().orc_matvec(self.h, _p(d), _p(out))
        return out

    def jacobi_diagonal(self):
        out = self._vec(3 * self.n_free)
        self.lib().orc_jacobi_diagonal(self.h, _p(out))
        return out

    def element_stress(self):
        out = self._vec(9 * self.n_tets)
        self.lib().orc_element_stress(self.h, _p(out))
        return out.reshape(-1, 3, 3)

    def element_forces(self):
        out = self._vec(12 * self.n_tets)
        self.lib().orc_element_forces(self.h, _p(out))
        return out.reshape(-1, 4, 3)

    def elastic_energy(self):
        return self.lib().orc_elastic_energy(self.h)

    def total_energy(self):
        return self.lib().orc_total_energy(self.h)

    def count_inverted(self):
        return self.lib().orc_count_inverted(self.h)

    def force_param_grads(self):
        a, b, c = self._vec(3 * self.n_free), self._vec(3 * self.n_free), self._vec(3 * self.n_free)
        self.lib().orc_force_param_grads(self.h, _p(a), _p(b), _p(c))
        return a, b, c

    def pcg(self, b, diag=None, tol=1e-8, max_iters=10000):
        b = _f64(b)
        x = self._vec(b.size)
        rr = np.zeros(1)
        d = _p(_f64(diag)) if diag is not None else None
        if diag is not None:
            self._diag = _f64(diag)
            d = _p(self._diag)
        its = self.lib().orc_pcg(self.h, _p(b), _p(x), d, tol, max_iters, _p(rr))
        return x, its, rr[0]

    def newton_pcg(self, rtol=1e-8, max_newton=50, max_cg=100000, eta_max=0.5, eta_min=1e-10):
        st = np.zeros(4)
        status = self.lib().orc_newton_pcg(self.h, rtol, max_newton, max_cg, eta_max, eta_min, _p(st))
        return status, dict(newton_iters=int(st[0]), cg_iters=int(st[1]), rel_res=st[2], r0=st[3])

    def adjoint(self, dLdu, young_e, tol=1e-12, max_cg=100000):
        dLdu = _f64(dLdu)
        ye = _f64(young_e)
        dLdE = self._vec(self.n_tets)
        dLdf = self._vec(3 * self.n_free)
        its = self.lib().orc_adjoint(self.h, _p(dLdu), _p(ye), tol, max_cg, _p(dLdE), _p(dLdf))
        return dLdE, dLdf, its

    @classmethod
    def num_threads(cls):
        return cls.lib().orc_num_threads()


class RefHarness:
    """The reference's own sources (compiled unmodified into oracle/_ref) behind
    oracle/ref_harness.cpp.  Available only where the reference tree exists."""

    _lib = None

    @classmethod
    def available(cls) -> bool:
        return os.path.isdir(REF_TREE) or os.path.exists(REF_SO)

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(REF_SO):
                build_ref()
            lib = C.CDLL(REF_SO)
            lib.ref_create.restype = C.c_void_p
            lib.ref_create.argtypes = [_dp, C.c_int, _ip, C.c_int, _ip, C.c_int, C.c_double, C.c_double,
                                       C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_double]
            lib.ref_destroy.argtypes = [C.c_void_p]
            for name in ["ref_num_bcs", "ref_num_free"]:
                getattr(lib, name).argtypes = [C.c_void_p]
                getattr(lib, name).restype = C.c_int
            for name in ["ref_reshuffle_map", "ref_tets"]:
                getattr(lib, name).argtypes = [C.c_void_p, _ip]
            for name in ["ref_set_nodal_loads", "ref_set_positions_shuffled", "ref_get_positions_shuffled",
                         "ref_get_positions", "ref_compute_gradients", "ref_jacobi_diagonal",
                         "ref_element_stress"]:
                getattr(lib, name).argtypes = [C.c_void_p, _dp]
            lib.ref_set_force_fraction.argtypes = [C.c_void_p, C.c_double]
            lib.ref_set_pressure_surface.argtypes = [C.c_void_p, _ip, C.c_int, C.c_double]
            lib.ref_matvec.argtypes = [C.c_void_p, _dp, _dp]
            lib.ref_elastic_energy.argtypes = [C.c_void_p]
            lib.ref_elastic_energy.restype = C.c_double
            lib.ref_force_param_grads.argtypes = [C.c_void_p, _dp, _dp, _dp]
            lib.ref_step.argtypes = [C.c_void_p]
            lib.ref_set_sim.argtypes = [C.c_void_p, C.c_int, C.c_int]
            lib.ref_assemble_dense.argtypes = [C.c_void_p, _dp]
            lib.ref_set_time_step.argtypes = [C.c_void_p, C.c_double]
            lib.ref_step_dt.argtypes = [C.c_void_p, C.c_double]
            for name in ["ref_set_velocities_shuffled", "ref_get_velocities_shuffled", "ref_set_start_shuffled"]:
                getattr(lib, name).argtypes = [C.c_void_p, _dp]
            lib.ref_newton_direct.argtypes = [C.c_void_p, C.c_int, C.c_double, _dp]
            lib.ref_newton_direct.restype = C.c_int
            lib.ref_newton_fd.argtypes = [C.c_void_p, C.c_int, C.c_double, _dp]
            lib.ref_newton_fd.restype = C.c_int
            lib.ref_newton_ls_trace.argtypes = [C.c_void_p, C.c_int, C.c_double, _ip, _dp, _dp, C.c_int, _dp, _ip]
            lib.ref_newton_ls_trace.restype = C.c_int
            cls._lib = lib
        return cls._lib

    def __init__(self, nodes, tets, fixed, young, poisson, density=1070.0, gravity=0.0, zup=True,
                 material=MMT_NEO_HOOKEAN, solver=1, outer_iters=10, inner_iters=100, abs_tol=0.1):
        lib = self.lib()
        self.nodes = _f64(nodes)
        self.tets_in = _i32(tets)
        self.fixed = _i32(fixed)
        self.n_nodes = self.nodes.shape[0]
        self.n_tets = self.tets_in.shape[0]
        self.h = lib.ref_create(_p(self.nodes), self.n_nodes, _p(self.tets_in, _ip), self.n_tets,
                                _p(self.fixed, _ip), self.fixed.size, young, poisson, density, gravity,
                                int(zup), material, solver, outer_iters, inner_iters, abs_tol)
        self.n_bcs = lib.ref_num_bcs(self.h)
        self.n_free = lib.ref_num_free(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib().ref_destroy(self.h)
            self.h = None

    def _vec(self, n):
        return np.zeros(n, dtype=np.float64)

    def reshuffle_map(self):
        m = np.zeros(self.n_nodes, dtype=np.int32)
        self.lib().ref_reshuffle_map(self.h, _p(m, _ip))
        return m

    def tets(self):
        t = np.zeros((self.n_tets, 4), dtype=np.int32)
        self.lib().ref_tets(self.h, _p(t, _ip))
        return t

    def set_force_fraction(self, f):
        self.lib().ref_set_force_fraction(self.h, f)

    def set_nodal_loads(self, f):
        f = _f64(f)
        self.lib().ref_set_nodal_loads(self.h, _p(f))

    def set_pressure_surface(self, tris, pressure):
        self._tris = _i32(tris)
        self.lib().ref_set_pressure_surface(self.h, _p(self._tris, _ip), self._tris.shape[0], pressure)

    def set_positions_shuffled(self, x):
        x = _f64(x)
        self.lib().ref_set_positions_shuffled(self.h, _p(x))

    def positions_shuffled(self):
        x = self._vec(3 * self.n_nodes)
        self.lib().ref_get_positions_shuffled(self.h, _p(x))
        return x.reshape(-1, 3)

    def positions(self):
        x = self._vec(3 * self.n_nodes)
        self.lib().ref_get_positions(self.h, _p(x))
        return x.reshape(-1, 3)

    def gradients(self):
        r = self._vec(3 * self.n_free)
        self.lib().ref_compute_gradients(self.h, _p(r))
        return r

    def matvec(self, d):
        d = _f64(d).ravel()
        out = self._vec(3 * self.n_free)
        self.lib().ref_matvec(self.h, _p(d), _p(out))
        return out

    def jacobi_diagonal(self):
        out = self._vec(3 * self.n_free)
        self.lib().ref_jacobi_diagonal(self.h, _p(out))
        return out

    def element_stress(self):
        out = self._vec(9 * self.n_tets)
        self.lib().ref_element_stress(self.h, _p(out))
        return out.reshape(-1, 3, 3)

    def elastic_energy(self):
        return self.lib().ref_elastic_energy(self.h)

    def force_param_grads(self):
        a, b, c = self._vec(3 * self.n_free), self._vec(3 * self.n_free), self._vec(3 * self.n_free)
        self.lib().ref_force_param_grads(self.h, _p(a), _p(b), _p(c))
        return a, b, c

    def step(self):
        self.lib().ref_step(self.h)

    def assemble_dense(self):
        n = 3 * self.n_free
        K = np.zeros((n, n))
        self.lib().ref_assemble_dense(self.h, _p(K))
        return K

    # ---- dynamics (reshuffled node order) ----
    def set_sim(self, simtype, substeps=1):
        self.lib().ref_set_sim(self.h, int(simtype), int(substeps))

    def set_time_step(self, dt):
        self.lib().ref_set_time_step(self.h, float(dt))

    def set_velocities_shuffled(self, v):
        v = _f64(v).reshape(-1, 3)
        self.lib().ref_set_velocities_shuffled(self.h, _p(v))

    def velocities_shuffled(self):
        v = np.zeros((self.n_nodes, 3))
        self.lib().ref_get_velocities_shuffled(self.h, _p(v))
        return v

    def set_start_shuffled(self, x):
        x = _f64(x).reshape(-1, 3)
        self.lib().ref_set_start_shuffled(self.h, _p(x))

    def step_dt(self, dt):
        self.lib().ref_step_dt(self.h, float(dt))

    def newton_fd(self, max_iters=50, rel_tol=1e-12):
        r = np.zeros(1)
        it = self.lib().ref_newton_fd(self.h, max_iters, rel_tol, _p(r))
        return it, r[0]

    def newton_direct(self, max_iters=50, rel_tol=1e-12):
        r = np.zeros(1)
        it = self.lib().ref_newton_direct(self.h, max_iters, rel_tol, _p(r))
        return it, r[0]

    def newton_ls_trace(self, max_iters=400, abs_tol=1e-9, cap=100000):
        """The reference's NewtonSolverBackTrack with its Bonet-Wood condition (SolveNewtonLS's set-up):
        per line-search trial the Newton iteration, the step length and the residual norm."""
        it = np.zeros(cap, dtype=np.int32)
        step = np.zeros(cap)
        res = np.zeros(cap)
        r0 = np.zeros(1)
        conv = np.zeros(1, dtype=np.int32)
        n = self.lib().ref_newton_ls_trace(self.h, max_iters, abs_tol, _p(it, _ip), _p(step), _p(res), cap,
                                           _p(r0), _p(conv, _ip))
        return dict(it=it[:n].copy(), step=step[:n].copy(), res=res[:n].copy(), r0=float(r0[0]),
                    converged=bool(conv[0]))
