"""TEST INFRASTRUCTURE ONLY: FP64 numpy restatement of a two-level (coarse-space) preconditioner
for the flexible-CG inner solves, the checker for a device implementation of it.  The reference
has no coarse space (its CG is Jacobi-preconditioned at most), so this oracle is pinned by its
own algebraic properties (tests/test_coarse_oracle.py), not by the reference.

Definition (free DOFs in the reshuffled order, 3 per node):
  aggregates: the free nodes grouped by the cell of a uniform grid (spacing `cell`) that holds
              their rest position
  P:          per aggregate, the six rigid-body modes of its nodes (three translations and three
              rotations about the aggregate's centroid), orthonormalised; modes that degenerate
              (an aggregate of one node or of collinear nodes) are dropped.  P^T P = I.
  Kc:         P^T K P (dense; symmetric positive definite when K is)
  M2(r):      M(r) + P Kc^-1 P^T r, M the one-level preconditioner (Jacobi or learned)
The tangent K is probed from the FP64 oracle's Hessian-vector product with one product per
(colour, component) of a distance-2 colouring of the free-node graph.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp


def node_graph(o) -> sp.csr_matrix:
    """Free-node adjacency (nodes sharing a tet, diagonal included), pattern only."""
    t = o.tets().astype(np.int64) - o.n_bcs
    rows = np.repeat(t, 4, axis=1).ravel()
    cols = np.tile(t, (1, 4)).ravel()
    keep = (rows >= 0) & (cols >= 0)
    A = sp.coo_matrix((np.ones(int(keep.sum())), (rows[keep], cols[keep])), shape=(o.n_free, o.n_free)).tocsr()
    A.sum_duplicates()
    A.data[:] = 1.0
    return A


def distance2_colouring(A: sp.csr_matrix) -> np.ndarray:
    """Greedy colouring in which no two nodes of a colour share a neighbour."""
    A2 = (A @ A).tocsr()
    colour = -np.ones(A.shape[0], dtype=np.int64)
    for i in range(A.shape[0]):
        used = set(colour[A2.indices[A2.indptr[i]:A2.indptr[i + 1]]].tolist())
        c = 0
        while c in used:
            c += 1
        colour[i] = c
    return colour


def probe_tangent(o) -> sp.csr_matrix:
    """K over the free DOFs at the oracle's current state (the matrix of its matvec)."""
    A = node_graph(o)
    colour = distance2_colouring(A)
    n = 3 * o.n_free
    rows, cols, vals = [], [], []
    for c in range(int(colour.max()) + 1):
        S = np.where(colour == c)[0]
        sub = A[:, S].tocoo()
        i, j = sub.row, S[sub.col]  # row node i meets exactly one column node j of this colour
        for k in range(3):
            d = np.zeros(n)
            d[3 * S + k] = 1.0
            y = o.matvec(d).reshape(-1, 3)
            for a in range(3):
                rows.append(3 * i + a)
                cols.append(3 * j + k)
                vals.append(y[i, a])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def aggregate_cells(X: np.ndarray, cell: float) -> np.ndarray:
    """Aggregate id per node: the grid cell of its position, numbered compactly."""
    g = np.floor((X - X.min(axis=0)) / cell).astype(np.int64)
    span = g.max(axis=0) + 1
    key = (g[:, 0] * span[1] + g[:, 1]) * span[2] + g[:, 2]
    _, aid = np.unique(key, return_inverse=True)
    return aid.ravel()


def rigid_body_basis(X: np.ndarray, aid: np.ndarray, rtol: float = 1e-8) -> sp.csr_matrix:
    """P: orthonormal rigid-body modes of every aggregate (columns grouped by aggregate)."""
    n = X.shape[0]
    na = int(aid.max()) + 1
    order = np.argsort(aid, kind="stable")
    starts = np.searchsorted(aid[order], np.arange(na + 1))
    rows, cols, vals = [], [], []
    ncol = 0
    for a in range(na):
        nodes = order[starts[a]:starts[a + 1]]
        d = X[nodes] - X[nodes].mean(axis=0)
        B = np.zeros((3 * nodes.size, 6))
        for c in range(3):
            B[c::3, c] = 1.0
        # rotation about axis e_r: e_r x d
        for r, (i, j) in enumerate(((1, 2), (2, 0), (0, 1))):
            B[i::3, 3 + r] = -d[:, j]
            B[j::3, 3 + r] = d[:, i]
        U, s, _ = np.linalg.svd(B, full_matrices=False)
        U = U[:, s > rtol * s[0]]
        dofs = (3 * nodes[:, None] + np.arange(3)).ravel()
        for c in range(U.shape[1]):
            rows.append(dofs)
            cols.append(np.full(dofs.size, ncol + c))
            vals.append(U[:, c])
        ncol += U.shape[1]
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(3 * n, ncol))


def coarse_matrix(K: sp.spmatrix, P: sp.spmatrix) -> np.ndarray:
    return np.asarray((P.T @ (K @ P)).todense())


def two_level(M, P: sp.spmatrix, Kc: np.ndarray):
    """r -> M(r) + P Kc^-1 P^T r (Kc factorised once)."""
    fac = sla.cho_factor(Kc)
    return lambda r: M(r) + P @ sla.cho_solve(fac, P.T @ r)


def fcg(K, b: np.ndarray, M, tol: float = 1e-8, max_it: int = 20000):
    """Flexible CG (Polak-Ribiere beta) for K x = b with preconditioner M: (x, iterations)."""
    x = np.zeros_like(b)
    r = b.copy()
    bn = np.linalg.norm(b)
    z = M(r)
    p = z.copy()
    rz = r @ z
    for it in range(1, max_it + 1):
        q = K @ p
        a = rz / (p @ q)
        x += a * p
        r_old = r.copy()
        r -= a * q
        if np.linalg.norm(r) <= tol * bn:
            return x, it
        z = M(r)
        beta = (z @ (r - r_old)) / rz
        rz = r @ z
        p = z + beta * p
    return x, max_it
