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
    m = 6 rigid-body modes ([I, -[d_i]x] R_a, ``sfem_coarse_factors``) or m = 12 affine modes
    ([I, L(d_i)] R_a with L's column 3 + 3 k + l giving component k the coordinate d_i[l],
    ``sfem_coarse_factors_affine``)."""
    if modes not in (6, 12):
        raise ValueError("modes is 6 (rigid) or 12 (affine)")
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)
    n = X.shape[0]
    lib = nat.load()
    aid = np.empty(n, dtype=np.int32)
    d = np.empty((n, 3), dtype=np.float64)
    na = C.c_int64()
    args = (X.ctypes.data_as(nat._dp), n, float(cell), float(rtol), aid.ctypes.data_as(nat._ip),
            d.ctypes.data_as(nat._dp))
    fn = lib.sfem_coarse_factors if modes == 6 else lib.sfem_coarse_factors_affine
    nat.check(fn(*args, None, C.byref(na)))
    R = np.empty((na.value, modes, modes), dtype=np.float64)
    nat.check(fn(*args, R.ctypes.data_as(nat._dp), C.byref(na)))
    return aid, d, R
