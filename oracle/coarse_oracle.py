"""TEST INFRASTRUCTURE ONLY: FP64 numpy restatement of a two-level (coarse-space) preconditioner
for the flexible-CG inner solves, the checker for a device implementation of it.  The reference
has no coarse space (its CG is Jacobi-preconditioned at most), so this oracle is pinned by its
own algebraic properties (tests/test_coarse_oracle.py), not by the reference.

Definition (free DOFs in the reshuffled order, 3 per node):
  aggregates: the free nodes grouped by the cell of a uniform grid (spacing `cell`) that holds
              their rest position
  P:          per aggregate, the six rigid-body modes of its nodes (three translations and three
              rotations about the aggregate's centroid), orthonormalised; modes that degenerate
              (an aggregate of one node or of collinear nodes) are dropped.  P^T P = I.  Compact
              form: node i's 3 x 6 block is B(d_i) R_a, d_i its offset from the centroid and
              R_a = diag(I / sqrt(n_a), W_a), W_a from the eigenpairs of the aggregate's inertia
              tensor (rigid_body_factors).
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
    """P: orthonormal rigid-body modes of every aggregate (columns grouped by aggregate), assembled
    from the compact form B(d_i) R_a of rigid_body_factors."""
    d, R = rigid_body_factors(X, aid, rtol)
    return basis_from_factors(aid, d, R)


def basis_from_factors(aid: np.ndarray, d: np.ndarray, R: np.ndarray) -> sp.csr_matrix:
    """P from a compact form: node i's block B(d_i) R_a, the nonzero columns of R_a kept in order
    (B the rigid-body modes for 6 x 6 factors, the affine ones for 12 x 12)."""
    kept = (np.abs(R).sum(axis=1) > 0).sum(axis=1)  # columns per aggregate
    first = np.concatenate([[0], np.cumsum(kept)])
    Bf = modes if R.shape[1] == 6 else (lambda dd: poly_modes(dd, 1 if R.shape[1] == 12 else 2))
    rows, cols, vals = [], [], []
    for i in range(d.shape[0]):
        a = aid[i]
        blk = Bf(d[i:i + 1]) @ R[a][:, :kept[a]]
        for c in range(3):
            rows.append(np.full(kept[a], 3 * i + c))
            cols.append(first[a] + np.arange(kept[a]))
            vals.append(blk[c])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                         shape=(3 * d.shape[0], int(first[-1])))


def modes(d: np.ndarray) -> np.ndarray:
    """B for nodes at offsets d from their centroid: (3 n x 6), translations then rotations."""
    B = np.zeros((3 * d.shape[0], 6))
    for c in range(3):
        B[c::3, c] = 1.0
    for r, (i, j) in enumerate(((1, 2), (2, 0), (0, 1))):
        B[i::3, 3 + r] = -d[:, j]
        B[j::3, 3 + r] = d[:, i]
    return B


def poly_modes(d: np.ndarray, degree: int) -> np.ndarray:
    """B of the polynomial modes for nodes at offsets d: (3 n x 3F), column F k + m giving component k
    the feature f_m(d) (poly_features)."""
    f = poly_features(d, degree)
    F = f.shape[1]
    B = np.zeros((3 * d.shape[0], 3 * F))
    for k in range(3):
        B[k::3, F * k:F * (k + 1)] = f
    return B


def rigid_body_factors(X: np.ndarray, aid: np.ndarray, rtol: float = 1e-8):
    """The compact form of P: per node its offset d_i from the aggregate's centroid, per aggregate a
    6 x 6 matrix R_a (zero columns for dropped modes) with P's block of node i = B(d_i) R_a.

    With the offsets summing to zero, B^T B = diag(n I, J), J = sum(|d|^2 I - d d^T) the
    aggregate's inertia tensor, so R_a = diag(I / sqrt(n), V L^-1/2) from the eigenpairs (L, V) of
    J; rotations whose eigenvalue is below rtol times the largest are dropped (one node: all three;
    collinear nodes: the one about their line)."""
    na = int(aid.max()) + 1
    cnt = np.bincount(aid, minlength=na).astype(np.float64)
    cen = np.zeros((na, 3))
    np.add.at(cen, aid, X)
    cen /= cnt[:, None]
    d = X - cen[aid]
    J = np.zeros((na, 3, 3))
    np.add.at(J, aid, (d * d).sum(axis=1)[:, None, None] * np.eye(3) - d[:, :, None] * d[:, None, :])
    R = np.zeros((na, 6, 6))
    R[:, :3, :3] = np.eye(3) / np.sqrt(cnt)[:, None, None]
    lam, V = np.linalg.eigh(J)  # ascending
    for a in range(na):
        keep = lam[a] > rtol * max(lam[a, -1], 0.0)
        k = int(keep.sum())
        R[a, 3:, 3:3 + k] = V[a][:, keep] / np.sqrt(lam[a][keep])
    return d, R


def poly_features(d: np.ndarray, degree: int) -> np.ndarray:
    """The node offsets' features (n x F): 1, dx, dy, dz (degree 1: F = 4), and dx^2, dy^2, dz^2,
    dx dy, dy dz, dz dx (degree 2: F = 10)."""
    f = [np.ones(len(d)), d[:, 0], d[:, 1], d[:, 2]]
    if degree == 2:
        f += [d[:, 0] ** 2, d[:, 1] ** 2, d[:, 2] ** 2, d[:, 0] * d[:, 1], d[:, 1] * d[:, 2], d[:, 2] * d[:, 0]]
    return np.stack(f, axis=1)


def poly_basis(X: np.ndarray, aid: np.ndarray, degree: int, rtol: float = 1e-3) -> sp.csr_matrix:
    """P of the polynomial coarse space: per aggregate and displacement component the features of the
    nodes' offsets from the centroid (degree 1: the twelve affine motions u = t + A d; degree 2: thirty
    modes), orthonormalised per aggregate from the eigenpairs of the features' Gram matrix (formed on
    d / the aggregate's largest |d|), features of eigenvalue <= rtol times the largest left out (1e-3:
    nearly dependent modes, e.g. a quadratic feature along a thin aggregate's short direction).  The
    correction P Kc^-1 P^T depends on the span only, so any orthonormal basis of it serves."""
    na = int(aid.max()) + 1
    cnt = np.bincount(aid, minlength=na).astype(np.float64)
    cen = np.zeros((na, 3))
    np.add.at(cen, aid, X)
    cen /= cnt[:, None]
    d = X - cen[aid]
    rows, cols, vals = [], [], []
    ncol = 0
    for a in range(na):
        idx = np.where(aid == a)[0]
        h = np.abs(d[idx]).max()
        f = poly_features(d[idx] / (h if h > 0 else 1.0), degree)
        lam, V = np.linalg.eigh(f.T @ f)
        keep = lam > rtol * max(lam[-1], 0.0)
        Q = f @ (V[:, keep] / np.sqrt(lam[keep]))  # orthonormal feature columns
        r_ = (3 * idx[:, None] + np.arange(3)[None, :]).ravel()
        for k in range(3):
            for j in range(Q.shape[1]):
                v = np.zeros((len(idx), 3))
                v[:, k] = Q[:, j]
                rows.append(r_)
                cols.append(np.full(len(r_), ncol))
                vals.append(v.ravel())
                ncol += 1
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(3 * len(X), ncol))


def coarse_matrix(K: sp.spmatrix, P: sp.spmatrix) -> np.ndarray:
    return np.asarray((P.T @ (K @ P)).todense())


def coarse_matrix_blocks(K: sp.spmatrix, aid: np.ndarray, d: np.ndarray, R: np.ndarray) -> np.ndarray:
    """Kc from the 3 x 3 blocks of K, the form a device assembly uses: every block K_ij adds
    B_i^T K_ij B_j (6 x 6) to the aggregate pair (a(i), a(j)); Kc_ab = R_a^T G_ab R_b over the kept
    columns (ordered as in basis_from_factors).  Dense in the aggregate pairs: for small cases."""
    Kb = K.tobsr(blocksize=(3, 3))
    na = R.shape[0]
    rows = np.repeat(np.arange(Kb.shape[0] // 3), np.diff(Kb.indptr))
    cols = Kb.indices
    B = np.stack([modes(d[k:k + 1]) for k in range(d.shape[0])])  # (n, 3, 6)
    contrib = np.einsum("kxi,kxy,kyj->kij", B[rows], Kb.data, B[cols])
    G = np.zeros((na, na, 6, 6))
    np.add.at(G, (aid[rows], aid[cols]), contrib)
    kept = (np.abs(R).sum(axis=1) > 0).sum(axis=1)
    first = np.concatenate([[0], np.cumsum(kept)])
    Kc = np.zeros((first[-1], first[-1]))
    for a in range(na):
        for b in range(na):
            if np.any(G[a, b]):
                Kc[first[a]:first[a + 1], first[b]:first[b + 1]] = (R[a][:, :kept[a]].T @ G[a, b]
                                                                     @ R[b][:, :kept[b]])
    return Kc


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
