"""torch.autograd binding of the static equilibrium solve and its adjoint.

    u = equilibrium_displacement(phys, young_e, f_free)

``young_e`` is the per-element Young's modulus (E,) and ``f_free`` the dead nodal
loads on the free nodes ((N_f, 3), reshuffled order), both float64 CUDA tensors.
The forward runs the library's globalised Newton-PCG solve (sfem_newton_solve);
the backward runs the hand-written adjoint (sfem_adjoint_dev): one Jacobi-PCG
solve K lambda = dL/du with the symmetric tangent at the equilibrium, then
dL/dE_e = lambda_e . f_int,e / E_e and dL/df = lambda.  (The reference has only
global force-parameter gradients, Source/ElasticEnergy.cpp:284-315; the per-element
adjoint is an extension.)  Torch is only the caller here: all arithmetic is in
the CUDA library.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _native as nat


def _stream_to_handle(phys):
    s = torch.cuda.current_stream(phys_device(phys))
    nat.check(phys._lib.sfem_set_stream(phys.handle, C.c_void_p(s.cuda_stream)))


def phys_device(phys):
    return torch.device("cuda", getattr(phys, "device", 0))


class StaticEquilibrium(torch.autograd.Function):
    @staticmethod
    def forward(ctx, young_e, f_free, phys, rest_free, solve_kw, adjoint_tol):
        assert young_e.dtype == torch.float64 and f_free.dtype == torch.float64
        young_e = young_e.contiguous()
        f_free = f_free.contiguous()
        _stream_to_handle(phys)
        lib, h = phys._lib, phys.handle
        nat.check(lib.sfem_set_element_youngs_dev(h, C.c_void_p(young_e.data_ptr())))
        nat.check(lib.sfem_set_nodal_loads_free_dev(h, C.c_void_p(f_free.data_ptr())))
        nat.check(lib.sfem_set_free_positions_dev(h, C.c_void_p(rest_free.data_ptr())))
        st = phys.newton_solve(**solve_kw)
        if st["status"] != 0:
            raise RuntimeError(f"equilibrium solve did not converge: {st}")
        pos = torch.empty_like(rest_free)
        nat.check(lib.sfem_get_free_positions_dev(h, C.c_void_p(pos.data_ptr())))
        ctx.phys = phys
        ctx.adjoint_tol = adjoint_tol
        ctx.save_for_backward(young_e, f_free, pos)
        return pos - rest_free

    @staticmethod
    def backward(ctx, grad_u):
        young_e, f_free, pos = ctx.saved_tensors
        phys = ctx.phys
        _stream_to_handle(phys)
        lib, h = phys._lib, phys.handle
        # restore the state of this forward (the handle may have been reused since)
        nat.check(lib.sfem_set_element_youngs_dev(h, C.c_void_p(young_e.data_ptr())))
        nat.check(lib.sfem_set_nodal_loads_free_dev(h, C.c_void_p(f_free.data_ptr())))
        nat.check(lib.sfem_set_free_positions_dev(h, C.c_void_p(pos.data_ptr())))
        g = grad_u.contiguous().to(torch.float64)
        dE = torch.empty_like(young_e)
        df = torch.empty_like(f_free)
        nat.check(lib.sfem_adjoint_dev(h, C.c_void_p(g.data_ptr()), ctx.adjoint_tol, 0, C.c_void_p(dE.data_ptr()),
                                       C.c_void_p(df.data_ptr())))
        return dE, df, None, None, None, None


def equilibrium_displacement(phys, young_e, f_free, solve_kw=None, adjoint_tol=1e-10):
    """Differentiable free-node displacement at static equilibrium (see module doc)."""
    kw = dict(rel_tol=1e-10, max_newton=50)
    kw.update(solve_kw or {})
    rest = torch.as_tensor(phys.rest_free_positions(), dtype=torch.float64, device=phys_device(phys))
    return StaticEquilibrium.apply(young_e, f_free, phys, rest, kw, adjoint_tol)
