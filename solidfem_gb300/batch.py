"""Batched solves of independent bodies in one handle (the 64-body batched workload).

The bodies are concatenated into one mesh (disjoint components) with per-element Lame
parameters; every kernel launch of the Newton-Krylov solve covers all of them, and the
library converges each body against its own initial residual, masking converged bodies
(include/sfem.h: sfem_set_instances).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .mesh import box_lattice
from .physics import FemPhysicsMatrixFree


@dataclass
class BodySpec:
    n: int          # hexes along x; the lattice is n x n/4 x n/4 on [0,L]x[0,L/4]x[0,L/4]
    young: float
    poisson: float


def c4_specs(count: int = 64, seed: int = 0):
    """n log-uniform in [8, 64] rounded to a multiple of 4, E log-uniform in [1e4, 1e6] Pa,
    nu uniform in [0.3, 0.48] (seeded)."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(8), np.log(64), size=count))
    n = np.clip(4 * np.round(n / 4), 8, 64).astype(int)
    E = np.exp(rng.uniform(np.log(1e4), np.log(1e6), size=count))
    nu = rng.uniform(0.3, 0.48, size=count)
    return [BodySpec(int(a), float(b), float(c)) for a, b, c in zip(n, E, nu)]


def lame(E, nu):
    return 0.5 * E / (1 + nu), E * nu / (1 + nu) / (1 - 2 * nu)


class BatchedBodies:
    """Union of bodies, each a clamped (x = 0) cantilever box of length L under gravity.

    The tip deflection of such a cantilever (square section L/4) relative to its length is
    about 24 rho g L / E, so for E down to 1e4 Pa the default L = 0.01 m keeps the softest
    bodies at a deflection of a quarter of their length (a metre-scale body of E = 1e4 Pa
    folds over under its own weight)."""

    def __init__(self, specs, precision="fp32", density=1070.0, gravity=(0.0, 0.0, -9.81), length=0.01):
        spacing = 0.5 * length
        self.spacing = spacing
        nodes, tets, fixed, mu, lam, offsets = [], [], [], [], [], [0]
        self.meshes = []
        base = 0
        for k, sp in enumerate(specs):
            m = box_lattice(sp.n, sp.n // 4, sp.n // 4, extent=(length, length / 4, length / 4))
            self.meshes.append(m)
            x = m.nodes.copy()
            x[:, 1] += spacing * k  # separate the bodies in space (patch locality only)
            nodes.append(x)
            tets.append(m.tets + base)
            fixed.append(m.face_nodes(0, 0) + base)
            a, b = lame(sp.young, sp.poisson)
            mu.append(np.full(m.n_tets, a))
            lam.append(np.full(m.n_tets, b))
            base += m.n_nodes
            offsets.append(base)
        self.specs = list(specs)
        self.nodes = np.concatenate(nodes)
        self.tets = np.concatenate(tets).astype(np.int32)
        self.fixed = np.concatenate(fixed).astype(np.int32)
        self.offsets = np.asarray(offsets, dtype=np.int64)
        ref_E, ref_nu = specs[0].young, specs[0].poisson
        self.phys = FemPhysicsMatrixFree(self.tets, self.nodes, self.fixed, young=ref_E, poisson=ref_nu,
                                         density=density, gravity=gravity, material=3, precision=precision)
        self.phys.set_element_lame(np.concatenate(mu), np.concatenate(lam))
        self.phys.set_instances(self.offsets)

    def solve(self, **newton_kw):
        st = self.phys.newton_solve(**newton_kw)
        rel, its = self.phys.instance_stats(len(self.specs))
        st["instance_rel_res"] = rel
        st["instance_newton_iters"] = its
        return st

    def displacement(self, k):
        x = self.phys.get_positions()
        a, b = self.offsets[k], self.offsets[k + 1]
        return x[a:b] - self.nodes[a:b]
