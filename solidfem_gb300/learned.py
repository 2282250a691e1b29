"""Learned graph-network preconditioner (extension; the reference has no learned part).

M(r) = D^-1/2 (c x + S^T S x), x = D^-1/2 r, with S a linear 3-layer message-passing
network of width 64 on the free-node mesh graph: a symmetric positive definite operator
for every choice of weights, so conjugate gradients stay convergent whatever the training
reached.  The network, its training and its inference all run in the CUDA library
(include/sfem.h, sfem_gnn_*); this module is the host-side handle: collect
residual/correction pairs from plain Jacobi-PCG solves, train with Adam, save and
load the weights (raw float32 blob + JSON metadata), and use it as the
preconditioner of the flexible-PCG Newton solve (precond=PC_LEARNED).
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from . import _native as nat

_fp = C.POINTER(C.c_float)


def num_params() -> int:
    n = C.c_int32()
    nat.check(nat.load().sfem_gnn_num_params(C.byref(n)))
    return n.value


class LearnedPreconditioner:
    """Attached to one FP32 ``FemPhysicsMatrixFree``; the weights can be moved between
    handles (the network is independent of the mesh size)."""

    WIDTH, LAYERS, FEATURES = 64, 3, 3

    def __init__(self, phys, seed: int = 0):
        if phys.precision != "fp32":
            raise ValueError("the learned preconditioner runs in FP32 handles")
        self.phys = phys
        self._lib = nat.load()
        nat.check(self._lib.sfem_gnn_init(phys.handle, int(seed)))
        self.n_params = num_params()

    # ---- weights ----
    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, dtype=np.float32)
        nat.check(self._lib.sfem_gnn_get_params(self.phys.handle, p.ctypes.data_as(_fp)))
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        nat.check(self._lib.sfem_gnn_set_params(self.phys.handle, p.ctypes.data_as(_fp)))

    def save(self, path: str, meta: dict | None = None) -> None:
        p = self.get_params()
        p.tofile(path)
        info = {"n_params": int(p.size), "width": self.WIDTH, "layers": self.LAYERS, "features": self.FEATURES,
                "dtype": "float32"}
        info.update(meta or {})
        with open(os.path.splitext(path)[0] + ".json", "w") as f:
            json.dump(info, f, indent=1)

    def load(self, path: str) -> None:
        self.set_params(np.fromfile(path, dtype=np.float32))

    def set_inference(self, mode: str) -> None:
        """'poly': the network folded into 3x3 polynomial coefficients (default, exact since S
        is linear); 'layers': the BF16 tensor-core layer kernels."""
        nat.check(self._lib.sfem_gnn_set_inference(self.phys.handle, {"poly": 0, "layers": 1}[mode]))

    def graph_form(self) -> tuple[str, int]:
        """How the polynomial passes read the neighbours: ('patterns', table entries) when nodes
        share neighbour-delta lists, else ('delta16', 0) or ('index32', 0)."""
        form, pat = C.c_int32(), C.c_int32()
        nat.check(self._lib.sfem_gnn_graph_form(self.phys.handle, C.byref(form), C.byref(pat)))
        return ("index32", "delta16", "patterns")[form.value], pat.value

    def set_batch(self, batch: int) -> None:
        """Pairs per Adam step (the gradient is averaged over them)."""
        nat.check(self._lib.sfem_gnn_set_batch(self.phys.handle, int(batch)))

    def set_loss(self, mode: str) -> None:
        """'energy': ||M(r) - e||_K^2 / (e.r);  'residual': ||K M(r) - r||^2 / (r.r)."""
        nat.check(self._lib.sfem_gnn_set_loss(self.phys.handle, {"energy": 0, "residual": 1}[mode]))

    # ---- inference / gradients ----
    def apply(self, r_free) -> np.ndarray:
        r = np.ascontiguousarray(r_free, dtype=np.float64).ravel()
        out = np.zeros_like(r)
        nat.check(self._lib.sfem_gnn_apply(self.phys.handle, r.ctypes.data_as(nat._dp), out.ctypes.data_as(nat._dp)))
        return out

    def loss_grad(self, r_free, e_free):
        r = np.ascontiguousarray(r_free, dtype=np.float64).ravel()
        e = np.ascontiguousarray(e_free, dtype=np.float64).ravel()
        loss = C.c_double()
        g = np.zeros(self.n_params, dtype=np.float32)
        nat.check(self._lib.sfem_gnn_loss_grad(self.phys.handle, r.ctypes.data_as(nat._dp), e.ctypes.data_as(nat._dp),
                                               C.byref(loss), g.ctypes.data_as(_fp)))
        return loss.value, g

    # ---- data and training ----
    def collect(self, b_free=None, every: int = 10, max_snaps: int = 20, rel_tol: float = 1e-6) -> int:
        n = C.c_int32()
        if b_free is None:
            bp = None
        else:
            self._b = np.ascontiguousarray(b_free, dtype=np.float64).ravel()
            bp = self._b.ctypes.data_as(nat._dp)
        nat.check(self._lib.sfem_gnn_collect(self.phys.handle, bp, every, max_snaps, rel_tol, C.byref(n)))
        return n.value

    def dataset_size(self) -> int:
        n = C.c_int32()
        nat.check(self._lib.sfem_gnn_dataset_size(self.phys.handle, C.byref(n)))
        return n.value

    def clear_dataset(self) -> None:
        nat.check(self._lib.sfem_gnn_clear_dataset(self.phys.handle))

    def train(self, steps: int, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        losses = np.zeros(steps, dtype=np.float32)
        nat.check(self._lib.sfem_gnn_train(self.phys.handle, steps, lr, seed, losses.ctypes.data_as(_fp)))
        return losses
