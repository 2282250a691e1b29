"""solidfem_gb300: GB300-native matrix-free nonlinear elasticity (SolidFEM's
FemPhysicsMatrixFree / NewtonSolver / NonlinearCG / ElasticEnergy path).

The compute path is the CUDA library behind include/sfem.h; this package is the
host-side binding (ctypes), mesh/load generators and the torch adjoint.
"""
from . import mesh  # noqa: F401
from ._native import (FP32, FP64, LSC_ARMIJO, LSC_ENGINEERING, LSC_RESIDUAL, MMT_COROTATIONAL,  # noqa: F401
                      MMT_LINEAR, MMT_NEO_HOOKEAN, MMT_STVK, PC_JACOBI, PC_LEARNED, PC_NONE, SfemError)
from .physics import FemPhysicsMatrixFree  # noqa: F401
from .pysolidfem import NonlinearFEM  # noqa: F401

__all__ = ["FemPhysicsMatrixFree", "NonlinearFEM", "SfemError", "mesh"]
