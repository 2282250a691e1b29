"""Benchmark: time to 1e-8 relative residual of the static nonlinear solve.

Workload (one "step" = one complete static solve from the rest configuration):
  box [0,4]x[0,1]x[0,1] as a 256x64x64 hex lattice, 6 tets per hex
  (1,085,825 nodes / 6,291,456 tets), interior nodes jittered U(-0.2h, 0.2h)
  (seed 0), compressible neo-Hookean E=1e5 Pa, nu=0.49, bottom face z=0 clamped,
  per-node normal traction on the top face drawn from N(0, 200 Pa), smoothed by a
  Gaussian of width 4h and rescaled to 200 Pa std (load seeds 10000 + step).
  Relative residual = |r(x_k)|_2 / |r(x_0)|_2 of the FP64-accurate nonlinear residual.

Arms (one JSON line each):
  default          the repository's fastest method on the GPU: inexact Newton with FP32 flexible-CG
                   inner solves preconditioned by the learned network plus a rigid-body coarse
                   space (set up once per mesh, outside the timed solves, like the network's
                   weights), the symmetric tangent assembled per Newton step as the operator, FP64
                   Newton residual and convergence test; the plain FP64 Jacobi-PCG GPU solve of the
                   same load is timed beside it, and the oracle's FP64 residual certifies the result.
  --impl reference the oracle's CPU port of the reference path (FP64 Jacobi-PCG Newton over
                   the reference's matrix-free products) on the host cores, extrapolated from
                   a bounded sample by the iteration counts of the same algorithm.

Timing: W untimed warm-up solves, then K timed solves bracketed by a barrier and
cudaStreamSynchronize, CUDA events on the library's stream, max over ranks.  The
workload's element data (~0.35 GB FP32, ~0.6 GB FP64) exceeds the 129 MB L2.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time-to-1e-8 residual: learned-PCG FP32 vs Jacobi-PCG FP64 (1 GB300); HBM GB/s"
DIMS = (256, 64, 64)
EXTENT = (4.0, 1.0, 1.0)
YOUNG, POISSON, DENSITY = 1e5, 0.49, 1070.0
REL_TOL = 1e-8
LOAD_SEED0 = 10000
WORKLOAD = ("256x64x64 hexes x 6 tets (1,085,825 nodes / 6,291,456 tets), jitter 0.2h, neo-Hookean E=1e5 "
            "nu=0.49, bottom face clamped, random top traction N(0,200 Pa) smoothed 4h; time to |r|/|r0| <= 1e-8")

# Iteration counts of the FP64 Jacobi-PCG Newton solve of this workload (load seed 10000)
# measured on a GB300 with this repository's FP64 path (5 Newton steps, 10,166 CG
# iterations, 6 residual evaluations, 35.3 s); the CPU arm multiplies its measured
# per-operation costs by them (same algorithm, same counts in exact arithmetic).
FP64_JACOBI_COUNTS = {"newton_iters": 5, "cg_iters": 10166, "residual_evals": 6}


HVP_DRAM_BYTES_PER_TET = 220.1e6 / 3145728  # k_patch_hvp<float, NH, DIR> (ncu, see the traffic note below)
# k_ssell_hvp<float, DIR> (symmetric tangent, 16-bit columns, mirror slots): ncu dram__bytes_read.sum +
# dram__bytes_write.sum on the 128x64x64 case, 196.95 + 10.41 MB per launch, against the 207.80 MB the
# launch streams (stored blocks x 38 B + lower entries x 6 B + free nodes x 48 B)
SELL_DRAM_PER_ALGO_BYTE = (196.95e6 + 10.41e6) / 207.797844e6


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:  # noqa: BLE001
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.samples = []
        self.stop = threading.Event()
        self.device = device
        self.t = threading.Thread(target=self.run, daemon=True)

    def run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                v = [x.strip() for x in out.stdout.strip().split(",")]
                if len(v) == 7:
                    self.samples.append(v)
            except Exception:  # noqa: BLE001
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_workload(dims=DIMS):
    from solidfem_gb300.mesh import box_lattice

    m = box_lattice(*dims, extent=EXTENT, jitter=0.2, seed=0)
    fixed = m.face_nodes(2, 0)
    return m, fixed


def loads_for(m, seed):
    from solidfem_gb300.mesh import random_top_traction

    return random_top_traction(m, seed=seed)


def dist_backend():
    """NCCL between GPU ranks; gloo where no GPU is visible (the host-side tests of the
    replica logic), or as SFEM_BENCH_BACKEND says."""
    b = os.environ.get("SFEM_BENCH_BACKEND")
    if b:
        return b
    import torch

    return "nccl" if torch.cuda.is_available() else "gloo"


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        if not dist.is_initialized():
            dist.init_process_group(dist_backend())
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(x, world):
    """Maximum over ranks (the job's time is the slowest replica's)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seeds(rank, warmup, steps):
    """Load seeds of one replica: every rank solves its own loads (10000 + 1000 rank + i), so
    N replicas do N times the work of one (weak scaling) with no data-path exchange."""
    return [LOAD_SEED0 + rank * 1000 + i for i in range(warmup + steps)]


# ---------------------------------------------------------------------------
# CPU arm (oracle port)
# ---------------------------------------------------------------------------
def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:  # noqa: BLE001
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:  # noqa: BLE001
        pass
    import platform

    return platform.machine()


def make_oracle(m, fixed):
    from oracle.oracle import Oracle

    return Oracle(m.nodes, m.tets, fixed, YOUNG, POISSON, DENSITY, (0.0, 0.0, 0.0), 3)


def shuffled(o, x):
    """Node array in the caller's order -> the oracle's reshuffled order."""
    out = np.zeros_like(x)
    out[o.reshuffle_map()] = x
    return out


def oracle_rel_res(o, m, f, positions):
    """|r(x)| / |r(x0)| of the oracle's FP64 residual (ComputeGradients semantics) at the given
    positions (caller's node order) under the nodal loads f."""
    o.set_nodal_loads(f)
    o.set_positions_shuffled(shuffled(o, m.nodes))
    r0 = float(np.linalg.norm(o.gradients()))
    o.set_positions_shuffled(shuffled(o, positions))
    return float(np.linalg.norm(o.gradients())) / r0


def cpu_sample(m, fixed, counts, its=20, o=None):
    """Time the oracle's FP64 operations on the full workload mesh on the host cores and
    extrapolate a Jacobi-PCG Newton solve with the given iteration counts."""
    from oracle.oracle import Oracle

    if o is None:
        o = make_oracle(m, fixed)
    o.set_nodal_loads(loads_for(m, LOAD_SEED0))
    o.set_positions_shuffled(shuffled(o, m.nodes))
    t = time.perf_counter()
    r = o.gradients()
    t_grad = time.perf_counter() - t
    t = time.perf_counter()
    diag = o.jacobi_diagonal()
    t_diag = time.perf_counter() - t
    t = time.perf_counter()
    o.pcg(r, diag=diag, tol=1e-30, max_iters=its)
    t_iter = (time.perf_counter() - t) / its
    est = (counts["cg_iters"] * t_iter + counts["newton_iters"] * t_diag + counts["residual_evals"] * t_grad)
    sample = (f"oracle port on {m.n_tets} tets: 1 residual ({t_grad:.2f} s, serial as the reference), "
              f"1 Jacobi diagonal ({t_diag:.2f} s), {its} PCG iterations measured ({t_iter:.3f} s/it, OpenMP "
              f"element loop); extrapolated x {counts['cg_iters']} CG its, {counts['newton_iters']} Newton its, "
              f"{counts['residual_evals']} residuals")
    return est, sample, Oracle.num_threads()


def run_reference_arm(args):
    rank, world, _ = dist_init()
    if rank != 0:
        return
    m, fixed = make_workload(DIMS if not args.small else (64, 16, 16))
    counts = dict(FP64_JACOBI_COUNTS)
    if counts["cg_iters"] is None:
        print(json.dumps({"impl": "reference", "unavailable": "iteration counts of the FP64 Jacobi-PCG solve "
                          "not recorded yet"}))
        return
    vals = []
    for _ in range(args.steps):
        est, sample, cores = cpu_sample(m, fixed, counts)
        vals.append(est)
    v = float(np.mean(vals))
    line = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": 0,
            "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD if not args.small else "reduced (64, 16, 16) variant of: " + WORKLOAD,
                       "method": "FP64 Jacobi-PCG Newton, oracle CPU port (extrapolated)"},
            "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port", "sample": sample,
                             "cpu_model": cpu_model()},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu_arm(args):
    import torch

    rank, world, local = dist_init()
    torch.cuda.set_device(local)
    from solidfem_gb300 import FemPhysicsMatrixFree

    dims = DIMS if not args.small else (64, 16, 16)
    if args.dims:
        dims = tuple(int(v) for v in args.dims.split(","))
    m, fixed = make_workload(dims)
    seeds = replica_seeds(rank, args.warmup, args.steps)
    loads = {s: loads_for(m, s) for s in seeds}
    kw = dict(young=YOUNG, poisson=POISSON, density=DENSITY, gravity=(0.0, 0.0, 0.0), material=3, device=local)
    solve_kw = dict(rel_tol=REL_TOL, max_newton=30, max_cg=200000)

    p32 = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, precision="fp32", **kw)
    p32.set_operator(args.operator)
    p32.set_residual_arithmetic(args.residual)
    method = "jacobi"
    coarse_setup_s = None
    coarse_info = None
    # the two-level method's network was fine-tuned with the coarse correction in the loop
    data = os.path.join(ROOT, "solidfem_gb300", "data")
    weights = args.weights if args.weights else os.path.join(data, "gnn_slab.bin")
    if not args.weights and args.coarse_cells > 0 and os.path.exists(os.path.join(data, "gnn_two_level.bin")):
        weights = os.path.join(data, "gnn_two_level.bin")
    if args.precond in ("learned", "auto") and os.path.exists(weights):
        from solidfem_gb300.learned import LearnedPreconditioner

        net = LearnedPreconditioner(p32)
        net.load(weights)
        method = "learned"
        if args.coarse_cells > 0:
            # two-level: the coarse space of cells of coarse_cells hexes, set up once per mesh
            # (rest-state tangent) like the network's weights, outside the timed solves
            t_cs = time.perf_counter()
            p32.set_coarse_space(args.coarse_cells * EXTENT[0] / dims[0], modes=args.coarse_modes)
            coarse_setup_s = time.perf_counter() - t_cs
            coarse_info = p32.coarse_info()
            method = "learned+coarse"
    elif args.precond == "learned":
        raise SystemExit(f"no trained weights at {weights}")
    from solidfem_gb300 import PC_JACOBI, PC_LEARNED

    main_pc = PC_LEARNED if method.startswith("learned") else PC_JACOBI
    rest = p32.get_free_positions()
    nf = p32.n_free
    # stage every step's inputs in HBM before the timed region (device-pointer API)
    dev_loads = {}
    mp = p32.reshuffle_map()
    for s in seeds:
        f = np.zeros((m.n_nodes, 3))
        f[mp] = loads[s]
        dev_loads[s] = torch.from_numpy(f[p32.n_bcs:].copy()).to(f"cuda:{local}")
    dev_rest = torch.from_numpy(rest.copy()).to(f"cuda:{local}")
    lib = p32._lib
    stream = torch.cuda.ExternalStream(_stream_of(p32))

    def solve(p, s, pc=None):
        lib.sfem_set_nodal_loads_free_dev(p.handle, dev_loads[s].data_ptr())
        lib.sfem_set_free_positions_dev(p.handle, dev_rest.data_ptr())
        return p.newton_solve(precond=main_pc if pc is None else pc, **solve_kw)

    for s in seeds[: args.warmup]:
        solve(p32, s)
    torch.cuda.synchronize()
    p32.set_profiling(True)
    l0 = FemPhysicsMatrixFree.kernel_launches()
    barrier(world)
    torch.cuda.synchronize()
    stats = []
    with ClockSampler(local) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for s in seeds[args.warmup:]:
            stats.append(solve(p32, s))
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = FemPhysicsMatrixFree.kernel_launches() - l0
    barrier(world)
    t_total = allmax(ev0.elapsed_time(ev1) / 1e3, world)
    value = t_total / args.steps
    prof = p32.get_profile()
    p32.set_profiling(False)
    ok = all(st["status"] == 0 and st["rel_res"] <= REL_TOL for st in stats)

    # end to end through the public host API: host loads in, positions out, every step
    e2e_t = None
    h2d = 8 * 3 * m.n_nodes
    d2h = 8 * 3 * m.n_nodes
    # inputs and the result in pinned host memory (torch's pinned allocator, viewed as numpy)
    pinned = {s: torch.from_numpy(loads[s]).pin_memory().numpy() for s in seeds[args.warmup:]}
    rest_full = torch.from_numpy(np.ascontiguousarray(m.nodes, dtype=np.float64)).pin_memory().numpy()
    out_pinned = torch.empty((m.n_nodes, 3), dtype=torch.float64).pin_memory().numpy()
    torch.cuda.synchronize()
    barrier(world)
    t = time.perf_counter()
    out = None
    for s in seeds[args.warmup:]:
        p32.set_nodal_loads(pinned[s])
        p32.set_positions(rest_full)
        p32.newton_solve(precond=main_pc, **solve_kw)
        out = p32.get_positions(out=out_pinned)
    torch.cuda.synchronize()
    e2e_t = allmax((time.perf_counter() - t) / args.steps, world)
    assert out is not None and np.isfinite(out).all()
    h2d += 8 * 3 * m.n_nodes  # rest positions sent each step

    pk, pk_kind = peaks()
    ms = prof["hvp_elem_ms"] / max(prof["samples"], 1)
    # algorithmic bytes of one FP32 Hessian-vector product: 56 B per tet (4 int32 corner indices,
    # Dm^-1 and the volume, as the reference stores them) + 36 B per node (x and p read, Kp written)
    algo_bytes = 56.0 * m.n_tets + 36.0 * m.n_nodes
    achieved = algo_bytes / (ms * 1e-3) / 1e9 if prof["samples"] else None
    # the bytes the launch itself must stream (for the assembled operator: the blocks, their columns
    # and per free node z, p_old in and p, q out), reported beside the unit above
    achieved_own = prof["algo_bytes_hvp"] / (ms * 1e-3) / 1e9 if prof["samples"] else None
    if args.operator == "assembled":
        kernel = ("k_ssell_hvp<float> (symmetric tangent assembled per Newton step: diagonal and upper blocks in "
                  "sliced ELL, lower blocks read transposed from their mirror rows)")
        # DRAM bytes per launch: an ncu capture of the 3,145,728-tet case, scaled by the streamed bytes
        traffic = args.traffic if args.traffic else SELL_DRAM_PER_ALGO_BYTE * prof["algo_bytes_hvp"]
        traffic_source = ("ncu capture at 3,145,728 tets scaled by the streamed bytes" if not args.traffic
                          else "--traffic")
    else:
        kernel = "k_patch_hvp<float, neo-Hookean> (fused element Hessian-vector product)"
        traffic = args.traffic if args.traffic else HVP_DRAM_BYTES_PER_TET * m.n_tets
        traffic_source = ("ncu capture at 3,145,728 tets scaled by the tet count" if not args.traffic
                          else "--traffic")

    # Jacobi-PCG FP32 of the first timed load (what the learned preconditioner replaces)
    s_ref = seeds[args.warmup]
    st_j32 = None
    if method.startswith("learned"):
        st_j32 = solve(p32, s_ref, PC_JACOBI)
    # the main method on the first timed load again: its equilibrium for the oracle and FP64 checks
    st_main = solve(p32, s_ref)
    x32 = p32.get_positions()
    # the same method through the matrix-free patch product (second record: the reference's operator form)
    mf = None
    if args.operator == "assembled" and not args.skip_matrix_free:
        p32.set_operator("matrix-free")
        solve(p32, s_ref)
        torch.cuda.synchronize()
        p32.set_profiling(True)
        mf_stats = [solve(p32, s_) for s_ in seeds[args.warmup:args.warmup + 2]]
        mprof = p32.get_profile()
        p32.set_profiling(False)
        mf_ms = mprof["hvp_elem_ms"] / max(mprof["samples"], 1)
        mf_ach = algo_bytes / (mf_ms * 1e-3) / 1e9 if mprof["samples"] else None
        mf = {"s_per_solve": [st_["seconds"] for st_ in mf_stats],
              "newton_iters": [st_["newton_iters"] for st_ in mf_stats],
              "cg_iters": [st_["cg_iters"] for st_ in mf_stats],
              "converged": all(st_["status"] == 0 and st_["rel_res"] <= REL_TOL for st_ in mf_stats),
              "kernel": "k_patch_hvp<float, neo-Hookean>", "ms_per_launch": mf_ms,
              "achieved_gbs": mf_ach, "frac": mf_ach / pk if mf_ach else None, "peak_source": pk_kind}
        p32.set_operator(args.operator)
    # plain FP64 Jacobi-PCG of the first timed load (the comparison the metric names)
    t64 = None
    st64 = None
    st64a = None
    x64 = None
    if not args.skip_fp64:
        p32.close()
        p64 = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, precision="fp64", **kw)
        torch.cuda.synchronize()
        st64 = solve(p64, s_ref, PC_JACOBI)
        t64 = st64["seconds"]
        x64 = p64.get_positions()
        # the same FP64 solve through the assembled FP64 operator (context; the metric's FP64 baseline
        # is the matrix-free solve above, the reference's method)
        p64.set_operator("assembled")
        solve(p64, s_ref, PC_JACOBI)  # builds the sliced-ELL structure once
        st64a = solve(p64, s_ref, PC_JACOBI)
        p64.close()

    # parity of the timed result: the oracle's FP64 residual (ComputeGradients semantics) at the
    # GPU's equilibria, and the FP32 solution's displacement error against the FP64 solve
    oracle = None
    parity = None
    if rank == 0 and not args.skip_oracle:
        oracle = make_oracle(m, fixed)
        parity = {"load_seed": s_ref,
                  "oracle_rel_res": oracle_rel_res(oracle, m, loads[s_ref], x32),
                  "oracle_rel_res_fp64_solve": (oracle_rel_res(oracle, m, loads[s_ref], x64)
                                                if x64 is not None else None)}
        if x64 is not None:
            parity["fp32_vs_fp64_displacement_rel_err"] = float(
                np.linalg.norm(x32 - x64) / np.linalg.norm(x64 - m.nodes))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {
                "workload": WORKLOAD if dims == DIMS else f"reduced {dims} variant of: " + WORKLOAD,
                "method": ("inexact Newton (Eisenstat-Walker), " +
                           {"learned": "learned-preconditioner flexible PCG",
                            "learned+coarse": "two-level (learned + " +
                                              {6: "rigid-body", 12: "affine", 30: "quadratic"}.get(
                                                  args.coarse_modes, str(args.coarse_modes)) +
                                              " coarse modes per aggregate) flexible PCG",
                            "jacobi": "Jacobi-PCG"}[method] +
                           " inner solves in FP32, FP64-accurate residual and convergence test"),
                "coarse_cells": args.coarse_cells if method == "learned+coarse" else None,
                "coarse_modes": args.coarse_modes if method == "learned+coarse" else None,
                "weights": os.path.basename(weights) if method.startswith("learned") else None,
                "coarse_setup_s": coarse_setup_s,
                "coarse_setup": coarse_info,
                "operator": args.operator,
                "residual_arithmetic": args.residual,
                "preconditioner": method, "l2": "inputs larger than L2 (element data 0.35 GB FP32)",
                "converged": ok, "newton_iters": [s_["newton_iters"] for s_ in stats],
                "cg_iters": [s_["cg_iters"] for s_ in stats],
                "parity": parity,
                "main_method_stats": st_main,
                "jacobi_fp32_stats": st_j32,
                "matrix_free": mf,
                "fp64_jacobi_pcg_s": t64,
                "fp64_jacobi_pcg_stats": st64,
                "fp64_jacobi_pcg_assembled_stats": st64a,
                "speedup_vs_fp64_jacobi": (t64 / value) if t64 else None,
                "solves_per_s_all_ranks": world * args.steps / t_total,
            },
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk, "unit": "GB/s",
                         "frac": achieved / pk if achieved else None, "traffic": traffic,
                         "kernel": kernel, "algo_bytes_per_launch": algo_bytes,
                         "algo_bytes_unit": "56 B per tet + 36 B per node (FP32 Hessian-vector product)",
                         "ms_per_launch": ms,
                         "streamed_bytes_per_launch": prof["algo_bytes_hvp"],
                         "achieved_on_streamed_bytes": achieved_own,
                         "frac_on_streamed_bytes": achieved_own / pk if achieved_own else None,
                         "peak_source": pk_kind, "traffic_source": traffic_source},
            "e2e": {"value": e2e_t, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "clocks": clk.summary(),
            "gpu_launches": launches,
        }
        if not args.skip_cpu and world == 1:
            counts = dict(FP64_JACOBI_COUNTS)
            if st64 is not None:
                counts = {"newton_iters": st64["newton_iters"], "cg_iters": st64["cg_iters"],
                          "residual_evals": st64["newton_iters"] + st64["line_search_cuts"] + 1}
            if counts["cg_iters"] is not None:
                est, sample, cores = cpu_sample(m, fixed, counts, o=oracle)
                line["cpu_baseline"] = {"value": est, "unit": "s", "cores": cores, "kind": "port",
                                        "sample": sample, "cpu_model": cpu_model()}
        print(json.dumps(line), flush=True)


def _stream_of(p):
    import ctypes as C

    s = C.c_void_p()
    p._lib.sfem_get_stream(p.handle, C.byref(s))
    return s.value


# ---------------------------------------------------------------------------
# The other configurations: GPU time beside the oracle port's CPU time (one JSON line each)
# ---------------------------------------------------------------------------
def _cpu_window(o, counts, its=20):
    """Per-operation CPU costs of the oracle port (one residual, one Jacobi diagonal, `its` PCG
    iterations, OpenMP over the host cores) extrapolated by a solve's operation counts."""
    t = time.perf_counter()
    r = o.gradients()
    t_grad = time.perf_counter() - t
    t = time.perf_counter()
    diag = o.jacobi_diagonal()
    t_diag = time.perf_counter() - t
    t = time.perf_counter()
    o.pcg(r, diag=diag, tol=1e-30, max_iters=its)
    t_iter = (time.perf_counter() - t) / its
    est = counts["cg_iters"] * t_iter + counts["newton_iters"] * t_diag + counts["residual_evals"] * t_grad
    return est, (f"measured: 1 residual {t_grad:.3f} s, 1 Jacobi diagonal {t_diag:.3f} s, {its} PCG iterations "
                 f"{t_iter * 1e3:.2f} ms/it; extrapolated x {counts['cg_iters']} CG its, {counts['newton_iters']} "
                 f"Newton its, {counts['residual_evals']} residuals")


def _gpu_newton(p, x0, reps=3, **kw):
    times, st = [], None
    for _ in range(reps + 1):
        p.set_positions(x0)
        st = p.newton_solve(**kw)
        times.append(st["seconds"])
    return float(np.median(times[1:])), st


def run_config(args):
    """C1 (16x4x4 cantilever, FP64 Newton to 1e-10), C2 (128x32x32, corotational and neo-Hookean,
    FP64 and FP32-refined to 1e-10), C4 (64 bodies, FP32-refined to 1e-8), C5 (64x16x16, per-element E:
    FP64 Newton to 1e-11 and the adjoint) on the GPU, next to the oracle port on the host cores."""
    import torch

    from oracle.oracle import Oracle
    from solidfem_gb300 import FemPhysicsMatrixFree
    from solidfem_gb300.mesh import box_lattice, lumped_face_load

    torch.cuda.init()
    cfg = args.config
    rec = {"metric": f"{cfg}: solve time, GPU beside the oracle CPU port", "config": cfg, "unit": "s"}
    cores = Oracle.num_threads()
    if cfg == "c1":
        m = box_lattice(16, 4, 4, extent=(4.0, 1.0, 1.0))
        fixed = m.face_nodes(0, 0)
        p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, young=1e5, poisson=0.45, density=1070.0,
                                 gravity=(0.0, 0.0, -9.81), material=3)
        t_gpu, st = _gpu_newton(p, m.nodes, rel_tol=1e-10, max_newton=200)
        o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, (0.0, 0.0, -9.81), 3)
        t = time.perf_counter()
        status, so = o.newton_pcg(rtol=1e-10, max_newton=200)
        t_cpu = time.perf_counter() - t
        rec.update(workload="16x4x4 x 6 tets (425 nodes / 1,536 tets), neo-Hookean E=1e5 nu=0.45, gravity, "
                            "FP64 Jacobi-PCG Newton to 1e-10",
                   gpu={"s": t_gpu, "newton_iters": st["newton_iters"], "cg_iters": st["cg_iters"],
                        "status": st["status"]},
                   cpu_baseline={"value": t_cpu, "kind": "port", "cores": cores, "cpu_model": cpu_model(),
                                 "sample": f"full solve measured (status {status}, {so['newton_iters']} Newton, "
                                           f"{so['cg_iters']} CG)"})
    elif cfg == "c2":
        m = box_lattice(128, 32, 32, extent=(8.0, 2.0, 2.0))
        fixed = m.face_nodes(0, 0)
        f = lumped_face_load(m, 0, 1, (0.0, 0.0, -500.0))
        rec["workload"] = ("128x32x32 x 6 tets (140,481 nodes / 786,432 tets), E=1e6 nu=0.4, 500 Pa -z traction "
                           "on x=8, Newton to 1e-10")
        for mat, name in ((2, "corotational"), (3, "neo-Hookean")):
            kw = dict(young=1e6, poisson=0.4, density=1070.0, gravity=(0, 0, 0), material=mat, tangent="exact")
            out = {}
            for prec in ("fp64", "fp32"):
                p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, precision=prec, **kw)
                p.set_nodal_loads(f)
                t_gpu, st = _gpu_newton(p, m.nodes, reps=1, rel_tol=1e-10, max_newton=60)
                out[prec] = {"s": t_gpu, "newton_iters": st["newton_iters"], "cg_iters": st["cg_iters"],
                             "status": st["status"]}
                if prec == "fp64":
                    counts = {"newton_iters": st["newton_iters"], "cg_iters": st["cg_iters"],
                              "residual_evals": st["newton_iters"] + st["line_search_cuts"] + 1}
                p.close()
            o = Oracle(m.nodes, m.tets, fixed, 1e6, 0.4, 1070.0, (0, 0, 0), mat)
            o.set_tangent(1)
            o.set_nodal_loads(f)
            est, sample = _cpu_window(o, counts)
            out["cpu_baseline"] = {"value": est, "kind": "port", "cores": cores, "cpu_model": cpu_model(),
                                   "sample": sample + " (the GPU FP64 solve's counts)"}
            rec[name] = out
    elif cfg == "c4":
        from solidfem_gb300.batch import BatchedBodies, c4_specs

        b = BatchedBodies(c4_specs(64, seed=0), precision="fp32")
        times = []
        for _ in range(3):
            b.phys.set_positions(b.nodes)
            st = b.solve(rel_tol=1e-8, max_newton=200)
            times.append(st["seconds"])
        rec.update(workload=f"64 bodies n x n/4 x n/4, n log-uniform [8,64] (seed 0), {b.phys.n_tets} tets, "
                            "FP32-refined Newton, every body to 1e-8",
                   gpu={"s": float(np.median(times[1:])), "newton_iters": st["newton_iters"],
                        "cg_iters": st["cg_iters"], "status": st["status"],
                        "max_body_rel_res": float(st["instance_rel_res"].max())})
        o = Oracle(b.nodes, b.tets, b.fixed, 1e5, 0.4, 1070.0, (0.0, 0.0, -9.81), 3)
        counts = {"newton_iters": st["newton_iters"], "cg_iters": st["cg_iters"],
                  "residual_evals": st["newton_iters"] + st["line_search_cuts"] + 1}
        est, sample = _cpu_window(o, counts)
        rec["cpu_baseline"] = {"value": est, "kind": "port", "cores": cores, "cpu_model": cpu_model(),
                               "sample": sample + " (FP64 per-operation cost on the union mesh, the GPU solve's "
                                                  "counts)"}
    elif cfg == "c5":
        m = box_lattice(64, 16, 16, extent=(4.0, 1.0, 1.0))
        fixed = m.face_nodes(0, 0)
        young = 1e5 * np.exp(0.5 * np.random.default_rng(1).normal(size=m.n_tets))
        f = lumped_face_load(m, 0, 1, (0.0, 0.0, -1000.0))
        p = FemPhysicsMatrixFree(m.tets, m.nodes, fixed, young=1e5, poisson=0.45, density=1070.0,
                                 gravity=(0.0, 0.0, 0.0), material=3)
        p.set_element_youngs(young)
        p.set_nodal_loads(f)
        t_gpu, st = _gpu_newton(p, m.nodes, rel_tol=1e-11, max_newton=100)
        dLdu = np.ones((p.n_free, 3))
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(3):
            p.adjoint(dLdu, rel_tol=1e-12)
        t_adj = (time.perf_counter() - t) / 3
        o = Oracle(m.nodes, m.tets, fixed, 1e5, 0.45, 1070.0, (0.0, 0.0, 0.0), 3)
        o.set_element_scale(young / 1e5)
        o.set_nodal_loads(f)
        counts = {"newton_iters": st["newton_iters"], "cg_iters": st["cg_iters"],
                  "residual_evals": st["newton_iters"] + st["line_search_cuts"] + 1}
        est, sample = _cpu_window(o, counts)
        o.set_free_positions(p.get_free_positions().ravel())
        t = time.perf_counter()
        _, _, its = o.adjoint(dLdu.ravel(), young, tol=1e-12, max_cg=200000)
        t_adj_cpu = time.perf_counter() - t
        rec.update(workload="64x16x16 x 6 tets (18,785 nodes / 98,304 tets), neo-Hookean nu=0.45, per-element E "
                            "log-normal (median 1e5, sigma 0.5), 1 kPa tip traction; FP64 Newton to 1e-11, adjoint "
                            "to 1e-12",
                   gpu={"newton_s": t_gpu, "newton_iters": st["newton_iters"], "cg_iters": st["cg_iters"],
                        "adjoint_s": t_adj},
                   cpu_baseline={"value": est + t_adj_cpu, "kind": "port", "cores": cores, "cpu_model": cpu_model(),
                                 "newton_s": est, "adjoint_s": t_adj_cpu,
                                 "sample": sample + f"; the adjoint solve measured in full ({its} PCG iterations)"})
    print(json.dumps(rec), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default=None, choices=["c1", "c2", "c4", "c5"],
                    help="time one of the other configurations (GPU beside the oracle CPU port) instead")
    ap.add_argument("--small", action="store_true", help="64x16x16 variant (quick check; not a bench line)")
    ap.add_argument("--dims", default=None, help="override the lattice, e.g. 128,64,64 (profiling; not a bench line)")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-oracle", action="store_true", help="no oracle residual at the GPU equilibria")
    ap.add_argument("--skip-matrix-free", action="store_true", help="no matrix-free record")
    ap.add_argument("--traffic", type=float, default=None, help="ncu dram bytes per HVP launch, if captured")
    ap.add_argument("--precond", default="auto", choices=["auto", "jacobi", "learned"],
                    help="auto: the learned preconditioner when trained weights exist, else Jacobi")
    ap.add_argument("--coarse-modes", type=int, default=30, choices=[6, 12, 30],
                    help="modes per coarse aggregate: 6 rigid-body, 12 affine, 30 quadratic")
    ap.add_argument("--coarse-cells", type=int, default=17,
                    help="two-level preconditioner with the learned one: coarse-space cells of this many hexes "
                         "per axis (0: the learned preconditioner alone)")
    ap.add_argument("--weights", default=None, help="trained weights (default solidfem_gb300/data/gnn_slab.bin)")
    ap.add_argument("--residual", default="two-term", choices=["two-term", "fp64"],
                    help="arithmetic of the FP32 solves' nonlinear residual: two-term FP32 (default, "
                         "FP64-accurate) or FP64 instructions")
    ap.add_argument("--operator", default="assembled", choices=["matrix-free", "assembled"],
                    help="operator of the FP32 Krylov solves: the tangent assembled per Newton step "
                         "(default, faster) or the matrix-free patch product; the FP64 baseline stays "
                         "matrix-free")
    args = ap.parse_args()
    if args.warmup < 3 and not args.small:
        args.warmup = 3
    if args.config:
        run_config(args)
    elif args.impl == "reference":
        run_reference_arm(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
