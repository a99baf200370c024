"""The multi-GPU path of bench.py on CPU: replicas over gloo, world size 2 (views shard with no exchange; the only
collective is the max over ranks of the timed region)."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms_local = [40.0, 55.0][rank]          # rank 1 is the slow one
    q.put((rank, bench.job_rate(ms_local, 1_000_000, world, dist, "cpu")))
    dist.destroy_process_group()


def test_job_rate_is_total_samples_over_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import socket

    mp = torch.multiprocessing.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    q = mp.Queue()
    ps = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        value, ms = out[r]
        assert ms == 55.0 and abs(value - 2_000_000 / 0.055 / 1e6) < 1e-9


def test_reference_arm_other_ranks_exit_without_work():
    env = {**os.environ, "RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
