"""The bench's multi-rank plumbing on CPU (gloo, world size 2): replicas only.

Each rank times its own replica; the job time is the max over ranks. The
reference arm runs on rank 0 only and the other ranks exit without work.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), HFX_BENCH_GLOO="1")
    sys.path.insert(0, ROOT)
    import bench
    w, r, _ = bench.dist_init()
    bench.barrier(w)
    q.put((r, bench.barrier_max(w, float(10 + r))))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_barrier_max_over_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert out == {0: 11.0, 1: 11.0}


def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ, HFX_BENCH_GLOO="1")
    port = 29700 + os.getpid() % 1000
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--config", "cfg1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"


def test_burgers_reference_arm_prints_its_metric():
    """The Burgers workload's reference arm (the oracle's HDGBurgersModel + Newton loop on
    a bounded sample) prints one line in the GPU arm's unit."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
           "--config", "burgers-small"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "elements*newton_iterations/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and "Newton" in d["cpu_baseline"]["sample"]


def test_anisotropic_lognormal_field():
    """The anisotropic lognormal coefficient of the 60^3x6 p=2 workload: exp(g) (I + 99 a a^T)
    per cell, g of standard deviation
    1.5, exactly symmetric and constant inside every cell (so the trace system is
    symmetric and the CG path applies)."""
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    cfg = bench.CONFIGS["cfg5-small"]
    coords, cells = bench.make_problem(cfg)
    k = bench.aniso_kappa(coords, cells, 3, **cfg["aniso"])
    assert k.shape == (cells.shape[0], cells.shape[1], 9)
    assert np.array_equal(k, np.broadcast_to(k[:, :1, :], k.shape))
    K = k[:, 0, :].reshape(-1, 3, 3)
    assert np.array_equal(K, np.swapaxes(K, 1, 2))
    ev = np.linalg.eigvalsh(K)
    assert np.allclose(ev[:, 2] / ev[:, 0], 100.0)
    g = np.log(ev[:, 0])
    assert abs(g.std() - 1.5) < 0.15 and abs(g.mean()) < 0.3


def test_batch_reference_arm_prints_its_metric():
    """The uneven batch's reference arm (the oracle, every sampled problem solved alone)
    prints one line in the GPU arm's unit."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
           "--config", "cfg3-small"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "elements/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and "each alone" in d["cpu_baseline"]["sample"]
