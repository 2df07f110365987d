"""The multi-rank path of bench.py (replicas: one independent lattice per
rank, no data-path collective; the slowest rank's time bounds the job) on
two CPU ranks over gloo, and the reference arm's rank guard."""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank builds its own replica of the workload (different seeded geometry)
        prm, g = bench.workload(64, 128, seed=bench.replica_seed(rank))
        digest = float(np.sum(g.mask_word.astype(np.int64) * np.arange(g.mask_word.size).reshape(g.mask_word.shape)))
        digests = bench.max_over_ranks([digest if r == rank else 0.0 for r in range(world)])
        # per-rank timings: the job time is the slowest rank's
        times = bench.max_over_ranks([10.0 + 5.0 * rank, 1.0 + rank])
        mlups = bench.job_mlups(world, 64 * 128, 100, times[0])
        if rank == 0:
            with open(out, "w") as fh:
                json.dump({"digests": digests, "times": times, "mlups": mlups}, fh)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "r.json")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    r = json.load(open(out))
    assert r["times"] == [15.0, 2.0]                       # max over ranks
    assert r["digests"][0] != r["digests"][1]               # independent replicas
    assert abs(r["mlups"] - 2 * 64 * 128 * 100 / 0.015 / 1e6) < 1e-6


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    p = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0 and p.stdout.strip() == ""
