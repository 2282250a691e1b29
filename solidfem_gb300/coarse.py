"""Coarse space of a two-level preconditioner, host side (``sfem_coarse_factors``): points grouped
into aggregates by the cells of a uniform grid, and each aggregate's orthonormal rigid-body basis
in compact form (per point its offset d_i from the aggregate's centroid, per aggregate a 6 x 6
matrix R_a; the point's 3 x 6 block of the basis is [I, -[d_i]x] R_a)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat


def coarse_factors(X, cell: float, rtol: float = 1e-8):
    """(aid, d, R) for the points X (n x 3): aggregate id per point (aggregates numbered in
    increasing cell order), offsets (n x 3) and R (n_agg x 6 x 6, zero columns for dropped
    rotations)."""
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)
    n = X.shape[0]
    lib = nat.load()
    aid = np.empty(n, dtype=np.int32)
    d = np.empty((n, 3), dtype=np.float64)
    na = C.c_int64()
    args = (X.ctypes.data_as(nat._dp), n, float(cell), float(rtol), aid.ctypes.data_as(nat._ip),
            d.ctypes.data_as(nat._dp))
    nat.check(lib.sfem_coarse_factors(*args, None, C.byref(na)))
    R = np.empty((na.value, 6, 6), dtype=np.float64)
    nat.check(lib.sfem_coarse_factors(*args, R.ctypes.data_as(nat._dp), C.byref(na)))
    return aid, d, R
