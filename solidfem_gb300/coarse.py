"""Coarse space of a two-level preconditioner, host side (``sfem_coarse_factors``): points grouped
into aggregates by the cells of a uniform grid, and each aggregate's orthonormal basis of rigid-body
(or affine) modes in compact form (per point its offset d_i from the aggregate's centroid, per
aggregate a 6 x 6 (12 x 12) matrix R_a; the point's 3 x 6 block of the basis is [I, -[d_i]x] R_a)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat


def coarse_factors(X, cell: float, rtol: float = 1e-8, modes: int = 6):
    """(aid, d, R) for the points X (n x 3): aggregate id per point (aggregates numbered in
    increasing cell order), offsets (n x 3) and R (n_agg x m x m, zero columns for dropped modes):
    m = 6 rigid-body modes ([I, -[d_i]x] R_a, ``sfem_coarse_factors``), or m = 12 / 30 polynomial modes
    of degree 1 / 2 (``sfem_coarse_factors_poly``: column F k + m of node i's block gives component k
    the feature f_m(d_i), F = m / 3)."""
    if modes not in (6, 12, 30):
        raise ValueError("modes is 6 (rigid), 12 (affine) or 30 (quadratic)")
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)
    n = X.shape[0]
    lib = nat.load()
    aid = np.empty(n, dtype=np.int32)
    d = np.empty((n, 3), dtype=np.float64)
    na = C.c_int64()
    args = (X.ctypes.data_as(nat._dp), n, float(cell), float(rtol))
    tail = (aid.ctypes.data_as(nat._ip), d.ctypes.data_as(nat._dp))
    if modes == 6:
        call = lambda R: lib.sfem_coarse_factors(*args, *tail, R, C.byref(na))
    else:
        call = lambda R: lib.sfem_coarse_factors_poly(*args, 1 if modes == 12 else 2, *tail, R, C.byref(na))
    nat.check(call(None))
    R = np.empty((na.value, modes, modes), dtype=np.float64)
    nat.check(call(R.ctypes.data_as(nat._dp)))
    return aid, d, R
