"""Synthetic box-lattice tetrahedral meshes and load fields.

Each hex of an nx x ny x nz lattice is split into 6 tetrahedra along its main
diagonal (the Kuhn/Freudenthal split: one tet per permutation of the axes), so
neighbouring hexes share face diagonals and the mesh is conforming.  Nodes are
numbered lexicographically with x fastest; every tet is emitted with positive
orientation (the reference's FemBody::Prepare would otherwise swap its first two
indices, Source/FemBody.cpp:127-156).

All generators are vectorised numpy and deterministic for a given seed.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass

import numpy as np

_PERMS = list(itertools.permutations(range(3)))


@dataclass
class BoxMesh:
    nodes: np.ndarray  # (N, 3) float64
    tets: np.ndarray  # (E, 4) int32
    dims: tuple  # (nx, ny, nz)
    extent: tuple  # (Lx, Ly, Lz)

    @property
    def n_nodes(self) -> int:
        return self.nodes.shape[0]

    @property
    def n_tets(self) -> int:
        return self.tets.shape[0]

    def node_index(self, i, j, k):
        nx, ny, _ = self.dims
        return i + (nx + 1) * (j + (ny + 1) * k)

    def face_nodes(self, axis: int, side: int) -> np.ndarray:
        """Indices of the nodes on the box face axis=min (side 0) or max (side 1)."""
        nx, ny, nz = self.dims
        n = (nx + 1, ny + 1, nz + 1)
        ii, jj, kk = np.meshgrid(np.arange(n[0]), np.arange(n[1]), np.arange(n[2]), indexing="ij")
        c = (ii, jj, kk)[axis]
        sel = c == (0 if side == 0 else n[axis] - 1)
        return np.sort(self.node_index(ii[sel], jj[sel], kk[sel]).astype(np.int32))

    def face_triangles(self, axis: int, side: int) -> np.ndarray:
        """Boundary triangles (T, 3) of one box face, as the Kuhn split cuts it:
        each quad is split along the diagonal joining its (0,0) and (1,1) corners."""
        nx, ny, nz = self.dims
        n = [nx, ny, nz]
        a, b = [d for d in range(3) if d != axis]
        fixed = 0 if side == 0 else n[axis]
        ua, ub = np.meshgrid(np.arange(n[a]), np.arange(n[b]), indexing="ij")
        ua = ua.ravel()
        ub = ub.ravel()

        def idx(da, db):
            c = [None, None, None]
            c[axis] = np.full_like(ua, fixed)
            c[a] = ua + da
            c[b] = ub + db
            return self.node_index(c[0], c[1], c[2])

        p00, p10, p01, p11 = idx(0, 0), idx(1, 0), idx(0, 1), idx(1, 1)
        t1 = np.stack([p00, p10, p11], axis=1)
        t2 = np.stack([p00, p01, p11], axis=1)
        return np.concatenate([t1, t2]).astype(np.int32)


def box_lattice(nx: int, ny: int, nz: int, extent=(1.0, 1.0, 1.0), jitter: float = 0.0,
                seed: int = 0) -> BoxMesh:
    """Kuhn 6-tet lattice of [0,Lx]x[0,Ly]x[0,Lz].  ``jitter`` moves every interior
    node by U(-jitter*h, jitter*h) per axis (h = the hex edge along that axis)."""
    Lx, Ly, Lz = extent
    xs = np.linspace(0.0, Lx, nx + 1)
    ys = np.linspace(0.0, Ly, ny + 1)
    zs = np.linspace(0.0, Lz, nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(np.float64)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        h = np.array([Lx / nx, Ly / ny, Lz / nz])
        kk, jj, ii = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
        interior = ((ii > 0) & (ii < nx) & (jj > 0) & (jj < ny) & (kk > 0) & (kk < nz)).ravel()
        d = rng.uniform(-jitter, jitter, size=(interior.sum(), 3)) * h
        nodes[interior] += d

    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i = i.ravel()
    j = j.ravel()
    k = k.ravel()

    def nid(di, dj, dk):
        return (i + di) + (nx + 1) * ((j + dj) + (ny + 1) * (k + dk))

    unit = np.eye(3, dtype=np.int64)
    tets = np.empty((i.size, 6, 4), dtype=np.int64)
    for t, perm in enumerate(_PERMS):
        c = np.zeros(3, dtype=np.int64)
        verts = [nid(*c)]
        for ax in perm:
            c = c + unit[ax]
            verts.append(nid(*c))
        # odd permutations have negative orientation: swap the first two vertices
        sign = np.linalg.det(np.stack([unit[perm[0]], unit[perm[1]], unit[perm[2]]]))
        if sign < 0:
            verts[0], verts[1] = verts[1], verts[0]
        tets[:, t, :] = np.stack(verts, axis=1)
    return BoxMesh(nodes=nodes, tets=tets.reshape(-1, 4).astype(np.int32), dims=(nx, ny, nz),
                   extent=(Lx, Ly, Lz))


def lumped_face_load(mesh: BoxMesh, axis: int, side: int, traction) -> np.ndarray:
    """Nodal forces (N, 3) of a uniform dead traction (Pa, 3-vector) on one box
    face, lumped as area/3 per boundary-triangle node."""
    tri = mesh.face_triangles(axis, side)
    p = mesh.nodes[tri]
    area = 0.5 * np.linalg.norm(np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), axis=1)
    w = np.zeros(mesh.n_nodes)
    for c in range(3):
        np.add.at(w, tri[:, c], area / 3.0)
    return w[:, None] * np.asarray(traction, dtype=np.float64)[None, :]


def nodal_face_area(mesh: BoxMesh, axis: int, side: int) -> np.ndarray:
    tri = mesh.face_triangles(axis, side)
    p = mesh.nodes[tri]
    area = 0.5 * np.linalg.norm(np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), axis=1)
    w = np.zeros(mesh.n_nodes)
    for c in range(3):
        np.add.at(w, tri[:, c], area / 3.0)
    return w


def _gauss_smooth_1d(a: np.ndarray, sigma: float, axis: int) -> np.ndarray:
    r = int(np.ceil(4 * sigma))
    x = np.arange(-r, r + 1)
    k = np.exp(-0.5 * (x / sigma) ** 2)
    k /= k.sum()
    pad = [(0, 0)] * a.ndim
    pad[axis] = (r, r)
    ap = np.pad(a, pad, mode="reflect")
    out = np.zeros_like(a)
    n = a.shape[axis]
    for t, w in enumerate(k):
        sl = [slice(None)] * a.ndim
        sl[axis] = slice(t, t + n)
        out += w * ap[tuple(sl)]
    return out


def random_top_traction(mesh: BoxMesh, seed: int, std: float = 200.0, sigma_h: float = 4.0) -> np.ndarray:
    """Nodal forces (N, 3) of a random normal (z) traction on the top face z=max.

    Per top node a magnitude is drawn from N(0, std), the field is smoothed by a
    normalised Gaussian of width ``sigma_h`` node spacings and rescaled to standard
    deviation ``std`` (Pa); each node gets traction * its lumped area."""
    nx, ny, _ = mesh.dims
    rng = np.random.default_rng(seed)
    w = rng.normal(0.0, std, size=(ny + 1, nx + 1))
    s = _gauss_smooth_1d(_gauss_smooth_1d(w, sigma_h, 0), sigma_h, 1)
    s *= std / max(s.std(), 1e-300)
    top = mesh.face_nodes(2, 1)  # sorted: x fastest, then y
    t = np.zeros(mesh.n_nodes)
    t[top] = s.ravel()
    area = nodal_face_area(mesh, 2, 1)
    f = np.zeros((mesh.n_nodes, 3))
    f[:, 2] = t * area
    return f
