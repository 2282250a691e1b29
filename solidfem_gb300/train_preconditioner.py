"""Train the learned preconditioner on residual/correction pairs from plain solves.

    python -m solidfem_gb300.train_preconditioner --out base.bin
    python -m solidfem_gb300.train_preconditioner --init base.bin --first-seed 128 --every 15 \
        --max-snaps 60 --lr 3e-4 --init-seed 1 --out tuned1.bin
    python -m solidfem_gb300.train_preconditioner --init tuned1.bin --first-seed 256 --every 15 \
        --max-snaps 60 --lr 1e-4 --init-seed 2 --out solidfem_gb300/data/gnn_slab.bin

The two-level preconditioner's network (the bench's default method) is the one-level network
fine-tuned on the corrections minus the coarse correction:

    python -m solidfem_gb300.train_preconditioner --init solidfem_gb300/data/gnn_slab.bin --coarse-cells 16 \
        --first-seed 512 --every 15 --max-snaps 60 --lr 3e-4 --init-seed 3 \
        --out solidfem_gb300/data/gnn_two_level.bin

Training meshes are slabs with the benchmark's element size (h = 1/64), jitter,
material (neo-Hookean E = 1e5 Pa, nu = 0.49) and boundary conditions (bottom face
clamped, random normal traction on the top face, load seeds 0..seeds-1).  For each
load the plain Jacobi-PCG solve of K x = r(x_0) on the GPU labels its own iterates:
(r_j, x_final - x_j) every `every` iterations.  The network is local (3 message-
passing hops), so weights trained on small slabs apply to the 256x64x64 mesh.
Training runs on the GPU (the library's BF16 tensor-core forward/backward kernels,
Adam on FP32 master weights, `batch` pairs per step).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import FemPhysicsMatrixFree
from .learned import LearnedPreconditioner
from .mesh import box_lattice, random_top_traction


def slab_mesh(nx, ny, nz, jitter=0.2, seed=0):
    return box_lattice(nx, ny, nz, extent=(nx / 64.0, ny / 64.0, nz / 64.0), jitter=jitter, seed=seed)


def train(dims=(64, 16, 16), seeds=128, every=25, max_snaps=40, steps=6000, lr=1e-3, init_seed=0, verbose=True,
          loss="energy", batch=16, init=None, first_seed=0, coarse_cells=0, coarse_modes=6):
    """Collect pairs from load seeds first_seed .. first_seed + seeds - 1 and train; init: weights
    to start from (a previous run's output) instead of the seeded random initialisation;
    coarse_cells > 0: train the network as the one-level part of the two-level preconditioner
    (coarse space of cells of that many hexes, coarse_modes modes per aggregate: 6 rigid, 12 affine, 30
    quadratic), i.e. on the corrections minus the coarse correction."""
    m = slab_mesh(*dims)
    fixed = m.face_nodes(2, 0)
    p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, young=1e5, poisson=0.49, density=1070.0, gravity=(0, 0, 0),
                             material=3, precision="fp32")
    net = LearnedPreconditioner(p, seed=init_seed)
    if init:
        net.load(init)
    if coarse_cells > 0:
        p.set_coarse_space(coarse_cells / 64.0, modes=coarse_modes)
    net.set_loss(loss)
    net.set_batch(batch)
    t0 = time.time()
    for s in range(first_seed, first_seed + seeds):
        p.set_nodal_loads(random_top_traction(m, seed=s))
        net.collect(None, every=every, max_snaps=max_snaps, rel_tol=1e-6)
    t_collect = time.time() - t0
    t0 = time.time()
    losses = net.train(steps=steps, lr=lr, seed=init_seed)
    t_train = time.time() - t0
    info = {"dims": list(dims), "load_seeds": [first_seed, first_seed + seeds - 1], "pairs": net.dataset_size(),
            "every": every, "max_snaps": max_snaps, "loss": loss, "batch": batch, "init": init, "init_seed": init_seed,
            "steps": steps, "lr": lr, "coarse_cells": coarse_cells, "coarse_modes": coarse_modes, "loss_first50": float(np.mean(losses[:50])),
            "loss_last50": float(np.mean(losses[-50:])), "collect_s": t_collect, "train_s": t_train,
            "material": "neo-Hookean E=1e5 nu=0.49, h=1/64, jitter 0.2h, bottom clamped, random top traction"}
    if verbose:
        print(json.dumps(info))
    return net, info, losses


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--dims", default="64,16,16")
    ap.add_argument("--seeds", type=int, default=128)
    ap.add_argument("--every", type=int, default=25)
    ap.add_argument("--max-snaps", type=int, default=40)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--loss", default="energy", choices=["energy", "residual"])
    ap.add_argument("--init", default=None, help="start from these weights (fine-tuning)")
    ap.add_argument("--first-seed", type=int, default=0, help="first load seed of the collected pairs")
    ap.add_argument("--init-seed", type=int, default=0, help="seed of the initialisation and of the minibatches")
    ap.add_argument("--coarse-cells", type=int, default=0,
                    help="train for the two-level preconditioner with coarse cells of this many hexes (0: one-level)")
    ap.add_argument("--coarse-modes", type=int, default=6, choices=[6, 12, 30], help="modes per coarse aggregate")
    a = ap.parse_args()
    dims = tuple(int(v) for v in a.dims.split(","))
    net, info, losses = train(dims, a.seeds, a.every, a.max_snaps, a.steps, a.lr, init_seed=a.init_seed, loss=a.loss,
                              batch=a.batch, init=a.init, first_seed=a.first_seed, coarse_cells=a.coarse_cells,
                              coarse_modes=a.coarse_modes)
    net.save(a.out, meta=info)
    np.save(a.out.rsplit(".", 1)[0] + "_losses.npy", losses)


if __name__ == "__main__":
    main()
