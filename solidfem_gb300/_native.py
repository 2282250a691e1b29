"""ctypes binding of the C ABI in include/sfem.h (libsfem_gb300.so).

The library is the only compute path: if it cannot be built or loaded this
module raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

SFEM_OK = 0
SFEM_NOT_CONVERGED = 1
SFEM_LINESEARCH_FAILED = 2
SFEM_ERR_INVALID = -1
SFEM_ERR_CUDA = -2
SFEM_ERR_NAN = -3
SFEM_ERR_INVERTED = -4
SFEM_ERR_OOM = -5
SFEM_ERR_BREAKDOWN = -6
SFEM_ERR_NO_DEVICE = -7
SFEM_ERR_TIMEOUT = -8

MMT_LINEAR, MMT_STVK, MMT_COROTATIONAL, MMT_NEO_HOOKEAN = 0, 1, 2, 3
# the other MaterialModelType values (FemDataStructures.h:93-107; FP64 handles)
(MMT_NEO_HOOKEAN_OGDEN, MMT_DISTORTIONAL_LINEAR, MMT_DISTORTIONAL_MOONEY, MMT_DISTORTIONAL_NH2, MMT_DISTORTIONAL_NH3,
 MMT_DISTORTIONAL_BW, MMT_DISTORTIONAL_OGDEN, MMT_DISTORTIONAL_NH6, MMT_DISTORTIONAL_NH7) = range(4, 13)
# materials whose reference energy is defined (ElasticEnergy.cpp:69-108): energy line searches apply
MATERIALS_WITH_ENERGY = (0, 1, 2, 3, 4, 6, 10)
FP64, FP32 = 0, 1
PC_NONE, PC_JACOBI, PC_LEARNED = 0, 1, 2
SIM_EXPLICIT, SIM_IMPLICIT = 2, 3
OP_MATRIX_FREE, OP_ASSEMBLED = 0, 1
RESIDUAL_FP64, RESIDUAL_TWO_TERM = 0, 1
LSC_ARMIJO, LSC_ENGINEERING, LSC_RESIDUAL = 0, 1, 2
TANGENT_REFERENCE, TANGENT_EXACT = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_vp = C.c_void_p


class Config(C.Structure):
    _fields_ = [("young", C.c_double), ("poisson", C.c_double), ("density", C.c_double),
                ("gravity", C.c_double * 3), ("material", C.c_int32), ("precision", C.c_int32),
                ("device", C.c_int32), ("tangent", C.c_int32)]


class PcgOpts(C.Structure):
    _fields_ = [("rel_tol", C.c_double), ("max_iters", C.c_int32), ("precond", C.c_int32),
                ("check_every", C.c_int32), ("reserved", C.c_int32)]


class PcgStats(C.Structure):
    _fields_ = [("iters", C.c_int32), ("status", C.c_int32), ("rel_res", C.c_double)]


class NewtonOpts(C.Structure):
    _fields_ = [("rel_tol", C.c_double), ("abs_tol", C.c_double), ("max_newton", C.c_int32),
                ("max_cg", C.c_int32), ("eta_max", C.c_double), ("eta_min", C.c_double),
                ("precond", C.c_int32), ("ls_condition", C.c_int32), ("max_bisection", C.c_int32),
                ("verbose", C.c_int32), ("load_steps", C.c_int32), ("reserved", C.c_int32)]


class NewtonStats(C.Structure):
    _fields_ = [("newton_iters", C.c_int32), ("cg_iters", C.c_int32), ("status", C.c_int32),
                ("line_search_cuts", C.c_int32), ("r0", C.c_double), ("rel_res", C.c_double),
                ("seconds", C.c_double)]


class Profile(C.Structure):
    _fields_ = [("hvp_elem_ms", C.c_double), ("hvp_gather_ms", C.c_double), ("samples", C.c_int64),
                ("hvp_launches", C.c_int64), ("algo_bytes_hvp", C.c_double), ("precision", C.c_int32),
                ("reserved", C.c_int32)]


class SfemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"sfem error {code}: {msg}")
        self.code = code


# (name, argtypes) of every exported entry point; restype is int unless noted
SIGNATURES = {
    "sfem_create": [_dp, C.c_int64, _ip, C.c_int64, _ip, C.c_int64, C.POINTER(Config), C.POINTER(_vp)],
    "sfem_destroy": [_vp],
    "sfem_last_error": [],
    "sfem_sizes": [_vp, _i64p, _i64p, _i64p],
    "sfem_reshuffle_map": [_vp, _ip],
    "sfem_get_stream": [_vp, C.POINTER(_vp)],
    "sfem_set_stream": [_vp, _vp],
    "sfem_get_positions": [_vp, _dp],
    "sfem_set_positions": [_vp, _dp],
    "sfem_get_free_positions": [_vp, _dp],
    "sfem_set_free_positions": [_vp, _dp],
    "sfem_set_lame_params": [_vp, C.c_double, C.c_double],
    "sfem_set_force_fraction": [_vp, C.c_double],
    "sfem_set_element_youngs": [_vp, _dp],
    "sfem_set_nodal_loads": [_vp, _dp],
    "sfem_set_pressure_surface": [_vp, _ip, C.c_int64, C.c_double],
    "sfem_set_element_lame": [_vp, _dp, _dp],
    "sfem_set_instances": [_vp, C.c_int32, _i64p],
    "sfem_instance_stats": [_vp, _dp, _ip],
    "sfem_compute_gradients": [_vp, _dp, _dp],
    "sfem_matvec": [_vp, _dp, _dp],
    "sfem_dot": [_vp, _dp, _dp, _dp],
    "sfem_jacobi_diagonal": [_vp, _dp],
    "sfem_energy": [_vp, _dp, _dp],
    "sfem_count_inverted": [_vp, _i64p],
    "sfem_element_stress": [_vp, _dp],
    "sfem_force_param_grads": [_vp, _dp, _dp, _dp],
    "sfem_pcg": [_vp, _dp, _dp, C.POINTER(PcgOpts), C.POINTER(PcgStats)],
    "sfem_newton_solve": [_vp, C.POINTER(NewtonOpts), C.POINTER(NewtonStats)],
    "sfem_tangent_nnz": [_vp, _i64p],
    "sfem_assemble_tangent": [_vp, _ip, _ip, _dp],
    "sfem_tangent_matvec": [_vp, _dp, _dp],
    "sfem_set_time_step": [_vp, C.c_double],
    "sfem_get_time_step": [_vp, _dp],
    "sfem_set_velocities": [_vp, _dp],
    "sfem_get_velocities": [_vp, _dp],
    "sfem_begin_step": [_vp],
    "sfem_step": [_vp, C.c_double, C.c_int32, C.c_int32, C.POINTER(NewtonOpts), C.POINTER(NewtonStats)],
    "sfem_nonlinear_cg": [_vp, C.c_int32, C.c_int32, C.c_double, _ip],
    "sfem_adjoint": [_vp, _dp, C.c_double, C.c_int32, _dp, _dp],
    "sfem_gnn_num_params": [_ip],
    "sfem_gnn_init": [_vp, C.c_uint64],
    "sfem_gnn_set_loss": [_vp, C.c_int32],
    "sfem_gnn_set_batch": [_vp, C.c_int32],
    "sfem_gnn_set_inference": [_vp, C.c_int32],
    "sfem_set_operator": [_vp, C.c_int32],
    "sfem_set_residual_arithmetic": [_vp, C.c_int32],
    "sfem_set_operator_memory_limit": [_vp, C.c_int64],
    "sfem_set_batched_pcg": [_vp, C.c_int32],
    "sfem_set_coarse_space": [_vp, C.c_double, C.c_double],
    "sfem_set_coarse_space_modes": [_vp, C.c_double, C.c_double, C.c_int32],
    "sfem_coarse_apply": [_vp, _dp, _dp],
    "sfem_coarse_info": [_vp, _ip, _ip, _dp],
    "sfem_instance_pcg_stats": [_vp, _ip, _ip, _dp],
    "sfem_set_device_wait": [_vp, C.c_int64, C.c_int32],
    "sfem_set_newton_trace": [_vp, _dp, C.c_int32, _ip],
    "sfem_operator_info": [_vp, _i64p, _ip],
    "sfem_gnn_graph_form": [_vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)],
    "sfem_coarse_factors": [_dp, C.c_int64, C.c_double, C.c_double, _ip, _dp, _dp, _i64p],
    "sfem_coarse_factors_poly": [_dp, C.c_int64, C.c_double, C.c_double, C.c_int32, _ip, _dp, _dp, _i64p],
    "sfem_gnn_get_params": [_vp, C.POINTER(C.c_float)],
    "sfem_gnn_set_params": [_vp, C.POINTER(C.c_float)],
    "sfem_gnn_apply": [_vp, _dp, _dp],
    "sfem_gnn_loss_grad": [_vp, _dp, _dp, _dp, C.POINTER(C.c_float)],
    "sfem_gnn_collect": [_vp, _dp, C.c_int32, C.c_int32, C.c_double, _ip],
    "sfem_gnn_dataset_size": [_vp, _ip],
    "sfem_gnn_clear_dataset": [_vp],
    "sfem_gnn_train": [_vp, C.c_int32, C.c_float, C.c_uint64, C.POINTER(C.c_float)],
    "sfem_set_profiling": [_vp, C.c_int32],
    "sfem_get_profile": [_vp, C.POINTER(Profile)],
    "sfem_kernel_launches": [_i64p],
    "sfem_dot_noalloc_dev": [_vp, _vp, C.c_int64, _vp, _vp],
    "sfem_compute_gradients_dev": [_vp, _vp],
    "sfem_matvec_dev": [_vp, _vp, _vp],
    "sfem_get_free_positions_dev": [_vp, _vp],
    "sfem_set_free_positions_dev": [_vp, _vp],
    "sfem_set_element_youngs_dev": [_vp, _vp],
    "sfem_set_nodal_loads_free_dev": [_vp, _vp],
    "sfem_adjoint_dev": [_vp, _vp, C.c_double, C.c_int32, _vp, _vp],
}

_lib = None
_lock = threading.Lock()


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the CUDA library; raises if unavailable."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_missing:
            try:
                _build.build(verbose=False)
            except Exception as e:  # noqa: BLE001 -- re-raised with context
                if not os.path.exists(_build.LIB):
                    raise ImportError(f"solidfem_gb300: CUDA library could not be built: {e}") from e
        if not os.path.exists(_build.LIB):
            raise ImportError(f"solidfem_gb300: {_build.LIB} missing; run `python -m solidfem_gb300.build`")
        lib = C.CDLL(_build.LIB)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = C.c_char_p if name == "sfem_last_error" else C.c_int
        _lib = lib
        return lib


def check(code: int, allow_positive: bool = True) -> int:
    if code < 0 or (code > 0 and not allow_positive):
        raise SfemError(code, load().sfem_last_error().decode())
    return code
