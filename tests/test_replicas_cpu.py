"""The multi-GPU form of the benchmark is replicas only (one independent solve per rank, no
data-path collective): its host logic -- rendezvous, barrier, max-over-ranks timing, per-rank
load seeds, and the reference arm printing once on rank 0 -- checked with world_size-2 gloo
process groups on CPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), SFEM_BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench

    r, w, _ = bench.dist_init()
    bench.barrier(w)
    t = bench.allmax(1.0 + r, w)
    seeds = bench.replica_seeds(r, 3, 2)
    out.put((r, w, t, seeds))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_barrier_max_and_seeds_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(k, 2, port, q)) for k in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[2] == 2.0 for r in res)  # the max over ranks reaches every rank
    assert len(set(res[0][3]) & set(res[1][3])) == 0  # every replica solves its own loads


@pytest.mark.timeout(600)
def test_reference_arm_prints_once_under_torchrun():
    port = _free_port()
    env = dict(os.environ, SFEM_BENCH_BACKEND="gloo", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference", "--small", "--steps", "1"]
    p = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["cpu_baseline"]["kind"] == "port"
